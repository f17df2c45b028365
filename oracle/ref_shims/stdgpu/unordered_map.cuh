// Test infrastructure (oracle side): project-written stand-in for
// stdgpu::unordered_map as torchhull uses it (marching_cubes_cuda.cu:66-70,
// 115-144, 184-212, 318-343, 725-810): integer keys (ravelled grid indices,
// never negative) mapped to integer values, filled by one kernel with
// emplace(), read by later kernels with find(), end() and it->second.
//
// Design: open addressing with linear probing over a power-of-two table of at
// least twice the requested capacity, keys claimed with a 64-bit atomicCAS.
// Every probe loop is bounded by the table size, so a full table ends the
// loop (emplace then reports failure, find returns end()); it never spins.
// end() is a real sentinel slot past the table whose value is 0, so a caller
// that dereferences end() reads index 0 instead of leaving the allocation.
// Which slot a key lands in does not affect torchhull's results: its outputs
// are ordered by the keys and indices themselves, not by the map's layout.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <type_traits>

#include <thrust/fill.h>

#include <stdgpu/memory.h>

namespace stdgpu
{

template <typename T1, typename T2>
struct pair
{
    T1 first;
    T2 second;
};

template <typename Key>
struct hash
{
    // SplitMix64 finaliser (Steele, Lea and Flood, "Fast splittable
    // pseudorandom number generators", 2014).
    __host__ __device__ std::uint64_t operator()(const Key& key) const
    {
        std::uint64_t z = static_cast<std::uint64_t>(key);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
};

template <typename Key>
struct equal_to
{
    __host__ __device__ bool operator()(const Key& a, const Key& b) const { return a == b; }
};

template <typename Key, typename T, typename Hash = hash<Key>, typename KeyEqual = equal_to<Key>,
          typename Allocator = std::allocator<pair<const Key, T>>>
class unordered_map
{
    static_assert(std::is_integral_v<Key> && sizeof(Key) == 8, "keys are 64-bit integers");

public:
    struct slot
    {
        Key first;
        T second;
    };
    using key_type = Key;
    using mapped_type = T;
    using iterator = slot*;
    using const_iterator = const slot*;
    using slot_allocator = typename std::allocator_traits<Allocator>::template rebind_alloc<slot>;

    // Keys are ravelled indices (>= 0), so -1 marks a free slot.
    static constexpr Key empty_key = Key(-1);

    unordered_map() = default;

    template <typename ExecutionPolicy>
    static unordered_map createDeviceObject(const ExecutionPolicy& policy, index_t capacity,
                                            const Allocator& allocator = Allocator())
    {
        unordered_map m;
        std::size_t size = 2;
        const std::size_t want = 2 * static_cast<std::size_t>(capacity > 0 ? capacity : 1);
        while (size < want)
        {
            size <<= 1;
        }
        slot_allocator alloc(allocator);
        m.slots_ = alloc.allocate(static_cast<index64_t>(size + 1));
        m.size_ = size;
        thrust::fill(policy, m.slots_, m.slots_ + size, slot{ empty_key, T{} });
        thrust::fill(policy, m.slots_ + size, m.slots_ + size + 1, slot{ empty_key, T{ 0 } });
        return m;
    }

    static void destroyDeviceObject(unordered_map& m)
    {
        if (m.slots_ != nullptr)
        {
            slot_allocator alloc{};
            alloc.deallocate(m.slots_, static_cast<index64_t>(m.size_ + 1));
            m.slots_ = nullptr;
            m.size_ = 0;
        }
    }

    __device__ pair<iterator, bool> emplace(const Key& key, const T& value)
    {
        const std::size_t mask = size_ - 1;
        std::size_t i = static_cast<std::size_t>(Hash{}(key)) & mask;
        for (std::size_t probe = 0; probe < size_; ++probe)
        {
            auto* word = reinterpret_cast<unsigned long long*>(&slots_[i].first);
            const unsigned long long prev = atomicCAS(word, static_cast<unsigned long long>(empty_key),
                                                      static_cast<unsigned long long>(key));
            if (prev == static_cast<unsigned long long>(empty_key))
            {
                slots_[i].second = value;
                return { &slots_[i], true };
            }
            if (KeyEqual{}(static_cast<Key>(prev), key))
            {
                return { &slots_[i], false };
            }
            i = (i + 1) & mask;
        }
        return { end(), false };
    }

    __device__ const_iterator find(const Key& key) const
    {
        const std::size_t mask = size_ - 1;
        std::size_t i = static_cast<std::size_t>(Hash{}(key)) & mask;
        for (std::size_t probe = 0; probe < size_; ++probe)
        {
            const Key k = slots_[i].first;
            if (KeyEqual{}(k, key))
            {
                return &slots_[i];
            }
            if (k == empty_key)
            {
                return end();
            }
            i = (i + 1) & mask;
        }
        return end();
    }

    __host__ __device__ const_iterator end() const { return slots_ + size_; }
    __host__ __device__ iterator end() { return slots_ + size_; }

private:
    slot* slots_ = nullptr;
    std::size_t size_ = 0;
};

} // namespace stdgpu
