// fsim_common.cuh -- device-side building blocks shared by the kernels of the
// step library (geometry of the padded MAC grid, particle buffers, reductions,
// counter-based random numbers).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fsim.h"

#include <mutex>
#include <set>
#include <utility>

// Raises a kernel's dynamic shared-memory limit on the current device, once per
// (kernel, device) and thread-safe; later calls only look the pair up.
inline cudaError_t set_smem_limit(const void* kern, int bytes) {
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({kern, dev})) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done.insert({kern, dev});
    return e;
}

#define FSIM_MAX_OBS 32
#define FSIM_DEAD_KEY 0xFFFFFFFFu

// Cell types (MacGridCell::CellType order).
#define C_WATER 0
#define C_AIR 1
#define C_SOLID 2

// Device error flags (OR-ed into ctx->d_err, read by the host after a step).
#define FSIM_DERR_TMA_TIMEOUT 1u
#define FSIM_DERR_NAN 2u

// Geometry of the padded grid.  Cells (x, y, z) with 0 <= z < nz are the
// reference's cells; storage pads z to pz (a multiple of 4 so every row starts
// on a 16-byte boundary, which the TMA tile loads require).  Linear index
// (x*ny + y)*pz + z.  Cells are cubes of edge h (3D grids only).
struct GridGeom {
    int nx, ny, nz, pz;
    long long ncell;   // nx * ny * pz
    float h, hinv;     // cellD.x = cellD.y
    double hd, hinvd;
    float hz, hzinv;   // cellD.z: h, or targetDimensions.z / 3 in 2D mode (macGrid.cpp:10)
    double hzd, hzinvd;
    double dims[3];    // MacGrid::dimensions
    int two_d;         // 2D mode: 3 cells in z, particles held at z = zc, no z motion
    float zc;          // HashedParticles::z = targetDimensions.z / 2 (simulationManager.cpp:27)
};

__host__ __device__ inline long long gidx(const GridGeom& g, int x, int y, int z) {
    return ((long long)x * g.ny + y) * g.pz + z;
}

// (x, y, z) of padded cell c in 32-bit arithmetic (64-bit division is emulated
// in software on the GPU; fsim_create keeps the padded grid below 2^31 cells)
__device__ __forceinline__ void cell_xyz(const GridGeom& g, long long c, int& x, int& y, int& z) {
    const unsigned cu = (unsigned)c, pz = (unsigned)g.pz, ny = (unsigned)g.ny;
    const unsigned t = cu / pz;
    z = (int)(cu - t * pz);
    const unsigned u = t / ny;
    y = (int)(t - u * ny);
    x = (int)u;
}

// SoA particle storage: 16 arrays of `cap` words each.
struct ParticleBuf {
    float* p[3];    // position
    float* v[3];    // velocity
    float* c[9];    // APIC vectors c[a] (row a = 3a..3a+2)
    uint32_t* id;   // stable particle id (optional)
};

// Obstacle as the kernels see it.  FP32 for the particle-side tests, FP64 for
// the grid rasterisation (which must match the reference's FP64 cell tests).
struct DevObstacle {
    int type;
    float pos[3], speed[3], size[3];
    float r;
    // push-out box bounds (MacGrid::getMinMaxRect +- particle radius)
    float box_lo[3], box_hi[3];
};

// ---- warp / block reductions -------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide reduction of K doubles (sum or max per slot, chosen by `is_max`
// bit k).  Result valid in thread 0.  `scratch` holds 32*K doubles.
template <int K>
__device__ __forceinline__ void block_reduce(double (&v)[K], unsigned is_max, double* scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = ((is_max >> k) & 1) ? warp_max(v[k]) : warp_sum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; k++) scratch[warp * K + k] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            double t = lane < nw ? scratch[lane * K + k] : (((is_max >> k) & 1) ? -1e300 : 0.0);
            v[k] = ((is_max >> k) & 1) ? warp_max(t) : warp_sum(t);
        }
    }
    __syncthreads();
}

// "Last block finishes": every block stores its partials, the block that
// arrives last reduces them all in block order (deterministic) and returns
// true in all of its threads.  partials: gridDim.x * K doubles.
template <int K>
__device__ __forceinline__ bool last_block_reduce(double (&v)[K], unsigned is_max, double* partials,
                                                  unsigned* counter, double* scratch) {
    __shared__ bool s_last;
    block_reduce<K>(v, is_max, scratch);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) partials[blockIdx.x * K + k] = v[k];
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; k++) acc[k] = ((is_max >> k) & 1) ? -1e300 : 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; k++) {
            double t = __ldcg(&partials[b * K + k]);
            acc[k] = ((is_max >> k) & 1) ? fmax(acc[k], t) : acc[k] + t;
        }
    block_reduce<K>(acc, is_max, scratch);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = acc[k];
        *counter = 0;
    }
    return true;
}

// ---- SplitMix64 (Steele, Lea, Flood 2014) as a counter-based generator -----
__host__ __device__ inline uint64_t splitmix64(uint64_t ctr) {
    uint64_t z = ctr * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ inline double uniform01(uint64_t seed, uint64_t i) {
    return (double)(splitmix64((seed << 32) + i + 1) >> 11) * (1.0 / 9007199254740992.0);
}

__host__ __device__ inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
