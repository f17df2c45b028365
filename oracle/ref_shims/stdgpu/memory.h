// Test infrastructure (oracle side): project-written stand-in for the part of
// stdgpu (commit d7c07d05, fetched by the reference's CMake build at
// _C/CMakeLists.txt:38-57) that torchhull's sources use, so that they compile
// unmodified without the stdgpu package.
//
// stdgpu's memory registration only feeds its own leak and bounds bookkeeping;
// torchhull allocates through torch's caching allocator
// (include/torchhull/stdgpu_allocator.h:36-49) and registers the blocks, so the
// registration calls here keep no record.
#pragma once

#include <cstddef>
#include <cstdint>

namespace stdgpu
{

using index64_t = std::ptrdiff_t;
using index_t = std::ptrdiff_t;

enum class dynamic_memory_type
{
    host,
    device,
    managed,
    invalid
};

template <typename T>
inline void register_memory(T* /*p*/, index64_t /*n*/, dynamic_memory_type /*type*/)
{
}

template <typename T>
inline void deregister_memory(T* /*p*/, index64_t /*n*/, dynamic_memory_type /*type*/)
{
}

// Tag for an empty device_unique_object.
struct null_object_t
{
};
inline constexpr null_object_t null_object{};

// Owns one device container created by T::createDeviceObject(policy, args...)
// and destroyed by T::destroyDeviceObject(object). Move-only.
template <typename T>
class device_unique_object
{
public:
    explicit device_unique_object(null_object_t) {}

    template <typename ExecutionPolicy, typename... Args>
    device_unique_object(const ExecutionPolicy& policy, Args&&... args)
        : object_(T::createDeviceObject(policy, static_cast<Args&&>(args)...)), owns_(true)
    {
    }

    device_unique_object(const device_unique_object&) = delete;
    device_unique_object& operator=(const device_unique_object&) = delete;

    device_unique_object(device_unique_object&& o) noexcept : object_(o.object_), owns_(o.owns_) { o.owns_ = false; }

    device_unique_object& operator=(device_unique_object&& o) noexcept
    {
        if (this != &o)
        {
            reset();
            object_ = o.object_;
            owns_ = o.owns_;
            o.owns_ = false;
        }
        return *this;
    }

    ~device_unique_object() { reset(); }

    T& operator*() { return object_; }
    const T& operator*() const { return object_; }
    T* operator->() { return &object_; }
    const T* operator->() const { return &object_; }

private:
    void reset()
    {
        if (owns_)
        {
            T::destroyDeviceObject(object_);
            owns_ = false;
        }
    }

    T object_{};
    bool owns_ = false;
};

} // namespace stdgpu
