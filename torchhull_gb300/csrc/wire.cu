// Candidate voxels as wireframes and curve networks as OBJ/PLY files
// (torchhull candidate_voxels_to_wireframes, visual_hull_cuda.cu:1022-1111;
// store_curve_network, io.cpp:11-127).

#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "th_internal.h"

namespace th
{
namespace
{

// The 12 cube edges as corner pairs (corner i = base + (i & 1, i >> 1 & 1,
// i >> 2 & 1)), in the order torchhull lists them
// (marching_cubes_table.h:335-338), so edge tensors match entry for entry.
__constant__ uint8_t kCubeEdges[12][2] = { { 0, 1 }, { 1, 5 }, { 4, 5 }, { 0, 4 }, { 2, 3 }, { 3, 7 },
                                           { 6, 7 }, { 2, 6 }, { 0, 2 }, { 1, 3 }, { 5, 7 }, { 4, 6 } };

// to_wireframe (visual_hull_cuda.cu:1024-1058): 8 corners and 12 edges per
// candidate of the level with resolution 2^shift.
__global__ void __launch_bounds__(256) wireframe_kernel(const int64_t* __restrict__ cand,
                                                       int64_t n,
                                                       int shift,
                                                       float cx,
                                                       float cy,
                                                       float cz,
                                                       float step,
                                                       float* __restrict__ verts,
                                                       int64_t* __restrict__ edges)
{
    const int64_t mask = (int64_t{ 1 } << shift) - 1;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        const int64_t id = cand[t];
        const int64_t gx = id & mask, gy = (id >> shift) & mask, gz = id >> (2 * shift);
#pragma unroll
        for (int i = 0; i < 8; ++i)
        {
            float* v = verts + 3 * (8 * t + i);
            v[0] = __fmaf_rn(step, static_cast<float>(gx + (i & 1)), cx);
            v[1] = __fmaf_rn(step, static_cast<float>(gy + ((i >> 1) & 1)), cy);
            v[2] = __fmaf_rn(step, static_cast<float>(gz + ((i >> 2) & 1)), cz);
        }
#pragma unroll
        for (int i = 0; i < 12; ++i)
        {
            edges[2 * (12 * t + i) + 0] = 8 * t + kCubeEdges[i][0];
            edges[2 * (12 * t + i) + 1] = 8 * t + kCubeEdges[i][1];
        }
    }
}

void write_obj(const std::string& filename, const float* verts, int64_t nv, const int64_t* edges, int64_t ne)
{
    std::ofstream file;
    file.open(filename);
    for (int64_t j = 0; j < nv; ++j)
        file << "v " << verts[3 * j] << " " << verts[3 * j + 1] << " " << verts[3 * j + 2] << "\n";
    for (int64_t j = 0; j < ne; ++j)
        file << "l " << 1 + edges[2 * j] << " " << 1 + edges[2 * j + 1] << "\n"; // 1-indexing
    file.close();
}

void write_ply(const std::string& filename, const float* verts, int64_t nv, const int64_t* edges, int64_t ne)
{
    std::ofstream file;
    file.open(filename);
    file << "ply\n";
    file << "format binary_little_endian 1.0\n";
    file << "element vertex " << nv << "\n";
    file << "property float x\n";
    file << "property float y\n";
    file << "property float z\n";
    file << "element edge " << ne << "\n";
    file << "property int vertex1\n";
    file << "property int vertex2\n";
    file << "end_header\n";
    file.close();
    std::ofstream bin(filename, std::ios::app | std::ios::binary);
    bin.write(reinterpret_cast<const char*>(verts), static_cast<std::streamsize>(sizeof(float) * 3 * nv));
    // int64 -> int32 as torch's .to(kInt) converts (two's-complement truncation); little endian
    std::vector<unsigned char> buf(static_cast<size_t>(8 * ne));
    for (int64_t j = 0; j < 2 * ne; ++j)
    {
        const uint32_t v = static_cast<uint32_t>(static_cast<uint64_t>(edges[j]));
        for (int b = 0; b < 4; ++b)
            buf[static_cast<size_t>(4 * j + b)] = static_cast<unsigned char>(v >> (8 * b));
    }
    bin.write(reinterpret_cast<const char*>(buf.data()), static_cast<std::streamsize>(buf.size()));
    bin.close();
}

} // namespace

void launch_wireframe(const int64_t* cand, int64_t n, int shift, const float corner[3], float length, float* verts, int64_t* edges, cudaStream_t s)
{
    if (n <= 0)
        return;
    // cube_length / float(2^shift), exact
    const float step = length / static_cast<float>(int64_t{ 1 } << shift);
    wireframe_kernel<<<grid_for(n, 256), 256, 0, s>>>(cand, n, shift, corner[0], corner[1], corner[2], step, verts,
                                                       edges);
    TH_LAUNCH_CHECK();
}

// The extension as std::filesystem::path::extension gives it ("" for none
// and for a leading dot of the file name).
std::string file_extension(const std::string& filename)
{
    const size_t dot = filename.find_last_of('.');
    const size_t slash = filename.find_last_of('/');
    const size_t name = slash == std::string::npos ? 0 : slash + 1;
    if (dot == std::string::npos || dot <= name)
        return std::string();
    return filename.substr(dot);
}

// store_curve_network (io.cpp:116-127): by extension, ".obj" text or ".ply"
// binary little endian; returns false for any other extension.
bool store_curve_network(const std::string& filename, const float* verts, int64_t nv, const int64_t* edges, int64_t ne, bool verbose)
{
    const std::string ext = file_extension(filename);
    if (ext != ".obj" && ext != ".ply")
        return false;
    if (verbose)
        std::cout << "Storing file \"" + filename + "\" ..." << std::endl;
    const auto t0 = std::chrono::high_resolution_clock::now();
    if (ext == ".obj")
        write_obj(filename, verts, nv, edges, ne);
    else
        write_ply(filename, verts, nv, edges, ne);
    const auto t1 = std::chrono::high_resolution_clock::now();
    const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0);
    if (verbose)
        std::cout << "Storing file \"" + filename + "\" ... done (" << static_cast<float>(ms.count()) / 1000.f << "s)"
                  << std::endl;
    return true;
}

} // namespace th
