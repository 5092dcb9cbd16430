// fsim_static.cu -- fsim_p2g_noalloc: the particle-to-grid transfer for
// callers that are not allowed to allocate GPU memory.
//
// Who needs it.  Some hosts of this library cannot call cudaMalloc at the time
// they want a transfer: a renderer or game loop that has a fixed frame budget
// (a device allocation can synchronise the whole device and stall the frame),
// an application that owns the GPU memory pool and hands plugins only the
// buffers it chose, or a pipeline that is recorded once and replayed.  The
// context API (fsim_create / fsim_step) allocates its buffers up front, which
// those callers cannot do.  This entry point runs the same cell sort and P2G
// kernels as FSIM_STAGE_P2G on buffers the caller owns, and keeps its only
// scratch -- per-particle cell keys, ranks and the sort permutation, per-cell
// counts and cell starts -- in one fixed array compiled into the library.
//
// That array is a file-scope __device__ variable, so every GPU on which the
// library's kernels are loaded holds its FSIM_NOALLOC_SCRATCH_BYTES until the
// process exits.  Host code cannot use the array's name as a device address;
// the first call on each device (with that device current) looks the address
// up with cudaGetSymbolAddress and caches it.  With CUDA's default lazy module
// loading that lookup is also where the library's module is loaded on the
// device and the array reserved -- an implicit device allocation that can
// synchronise the device -- so callers make their first call at set-up time
// (or run with CUDA_MODULE_LOADING=EAGER).
#include <cmath>
#include <mutex>

#include "fsim_ctx.h"

namespace {

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

constexpr size_t kMaxParticles = (size_t)FSIM_NOALLOC_MAX_PARTICLES;
constexpr size_t kMaxCells = (size_t)FSIM_NOALLOC_MAX_CELLS;
constexpr size_t kScanTile = 4096;  // items per scan tile (launch_scan)

constexpr size_t kOffKey = 0;
constexpr size_t kOffRank = kOffKey + align256(4 * kMaxParticles);
constexpr size_t kOffPerm = kOffRank + align256(4 * kMaxParticles);
constexpr size_t kOffCount = kOffPerm + align256(4 * kMaxParticles);
constexpr size_t kOffStart = kOffCount + align256(4 * (kMaxCells + 1));
constexpr size_t kOffBlocks = kOffStart + align256(4 * (kMaxCells + 1));
constexpr size_t kBytes = kOffBlocks + align256(4 * ((kMaxCells + 1 + kScanTile - 1) / kScanTile + 1));
static_assert(kBytes == (size_t)FSIM_NOALLOC_SCRATCH_BYTES, "scratch size in fsim.h is out of date");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
cudaError_t scratch_address(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_lock);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int fsim_p2g_noalloc(const fsim_grid_desc* grid, int transfer, const float* pos, const float* vel,
                                const float* c, int64_t n, float* vx, float* vy, float* vz, uint8_t* flags,
                                float* avg, void* stream) {
    if (!grid || !pos || !vel || !vx || !vy || !vz || !flags || !avg || n < 0) return FSIM_E_INVALID;
    if (transfer < FSIM_PIC || transfer > FSIM_APIC || (transfer == FSIM_APIC && !c)) return FSIM_E_INVALID;
    if (grid->two_d || !(grid->resolution > 0) || !std::isfinite(grid->resolution)) return FSIM_E_INVALID;
    // grid geometry as fsim_create derives it (MacGrid ctor, macGrid.cpp:9-13)
    GridGeom g{};
    g.hd = 1 / (double)(float)grid->resolution;
    g.hinvd = 1.0 / g.hd;
    g.h = (float)g.hd;
    g.hinv = (float)g.hinvd;
    g.hzd = g.hd;
    g.hzinvd = g.hinvd;
    g.hz = g.h;
    g.hzinv = g.hinv;
    // cells per axis, bounded in floating point before any integer conversion
    // (a product of three in-range axes can still wrap a 64-bit count)
    double cells_axis[3];
    for (int a = 0; a < 3; a++) {
        if (!std::isfinite(grid->dims[a]) || !(grid->dims[a] > 0)) return FSIM_E_INVALID;
        cells_axis[a] = std::floor(grid->dims[a] / g.hd);
        if (!(cells_axis[a] <= (double)kMaxCells)) return FSIM_E_CAPACITY;
    }
    if (!(cells_axis[0] * cells_axis[1] * cells_axis[2] <= (double)kMaxCells)) return FSIM_E_CAPACITY;
    g.nx = (int)cells_axis[0];
    g.ny = (int)cells_axis[1];
    g.nz = (int)cells_axis[2];
    if (g.nx < 3 || g.ny < 3 || g.nz < 3) return FSIM_E_INVALID;
    if (g.nz % 4 != 0) return FSIM_E_INVALID;  // outputs are dense: z rows must need no padding
    g.pz = g.nz;
    g.ncell = (long long)g.nx * g.ny * g.nz;
    for (int a = 0; a < 3; a++) g.dims[a] = (a == 0 ? g.nx : a == 1 ? g.ny : g.nz) * g.hd;
    if ((size_t)n > kMaxParticles || (size_t)g.ncell > kMaxCells) return FSIM_E_CAPACITY;
    // an error left pending by the caller's earlier work on this thread is
    // reported before anything is launched (and left pending), so that the
    // final launch check below reports only this call's launches
    if (cudaPeekAtLastError() != cudaSuccess) return FSIM_E_CUDA;

    unsigned char* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return FSIM_E_CUDA;
    uint32_t* key = reinterpret_cast<uint32_t*>(base + kOffKey);
    uint32_t* rank = reinterpret_cast<uint32_t*>(base + kOffRank);
    uint32_t* perm = reinterpret_cast<uint32_t*>(base + kOffPerm);
    int* count = reinterpret_cast<int*>(base + kOffCount);
    int* cstart = reinterpret_cast<int*>(base + kOffStart);
    int* blocks = reinterpret_cast<int*>(base + kOffBlocks);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // the counters keep the previous call's values: clear them first
    if (cudaMemsetAsync(count, 0, (size_t)g.ncell * sizeof(int), s) != cudaSuccess) return FSIM_E_CUDA;

    ParticleBuf p{};
    for (int a = 0; a < 3; a++) {
        p.p[a] = const_cast<float*>(pos) + (size_t)a * n;
        p.v[a] = const_cast<float*>(vel) + (size_t)a * n;
    }
    for (int k = 0; k < 9; k++) p.c[k] = c ? const_cast<float*>(c) + (size_t)k * n : nullptr;

    if (n > 0) {
        AdvectArgs a{};
        a.p = p;
        a.n = n;
        a.do_key = 1;
        a.g = g;
        a.key = key;
        a.rank = rank;
        a.count = count;
        launch_advect(a, s);
    }
    launch_scan(count, cstart, g.ncell, blocks, s);
    launch_scatter(key, rank, cstart, perm, n, g.ncell, s);
    float* const u[3] = {vx, vy, vz};
    if (launch_p2g_raw(p, perm, cstart, g, u, flags, avg, transfer == FSIM_APIC, s) != cudaSuccess)
        return FSIM_E_CUDA;
    return cudaGetLastError() == cudaSuccess ? FSIM_OK : FSIM_E_CUDA;
}
