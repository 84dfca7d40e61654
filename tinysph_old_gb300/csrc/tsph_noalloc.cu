// tsph_noalloc.cu -- Particle_To_Cell for callers that cannot allocate device
// memory.
//
// Some callers of this library cannot call cudaMalloc: a host framework that
// binds the library through its FFI and hands out device buffers only from its
// own pre-allocated pool, or a time loop that must not allocate because
// cudaMalloc / cudaFree synchronise the whole device.  They still own the
// particle positions and the output cell lists; what they cannot provide is
// the counting sort's working memory (cell counts, per-particle cells and
// slots, the scan's partial sums, the cell-index tables).  This file keeps
// that working memory in one file-scope device array, g_noalloc_scratch,
// sized for at most kNoAllocMaxParticles particles, kNoAllocMaxCells cells and
// kNoAllocMaxAxis cells per axis (about 16.1 MB, held by every GPU that loads
// the library until the process exits).  A cell may hold at most
// kNoAllocMaxPerCell particles: each particle's place in its cell is its rank
// among the cell's members, found by one pass over them, so a cell's cost
// grows with the square of its occupancy (SPH spacing puts about ten
// particles in a cell); a call with a fuller cell returns TSPH_ERR_ARG.
//
// Rules of use:
//  * The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and caches it; make the
//    first call on each device outside any stream capture.  The cached
//    address belongs to the device's current context: a caller that resets
//    the device (cudaDeviceReset) must not call this entry point again in
//    the same process.
//  * Every call shares the one array.  A call clears what must start at zero,
//    runs on the caller's stream and waits for it before returning; calls that
//    overlap on the GPU (e.g. from several host threads, or while another
//    stream still runs an earlier call's work) race on the array.  Calls made
//    through this entry point are serialised by a host mutex.
//  * The array keeps the last call's contents.
//  * Positions are read as two doubles per particle (8-byte alignment, the
//    alignment of any double array); misaligned pointers are refused before
//    anything is queued.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/tsph.h"
#include "tsph_engine.h"
#include "tsph_grid_host.h"
#include "tsph_kernels.cuh"

namespace {

constexpr int kNoAllocMaxParticles = 1 << 20;
constexpr int kNoAllocMaxCells = 1 << 20;
constexpr int kNoAllocMaxAxis = 8192;
constexpr int kNoAllocMaxDevices = 64;
constexpr int kNoAllocMaxPerCell = 4096;

// layout of the scratch array (byte offsets, each 256-byte aligned)
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCounts = 0;                                                  // u32[cells+1]
constexpr size_t kOffKey = align256(kOffCounts + 4 * ((size_t)kNoAllocMaxCells + 1));  // u32[n]
constexpr size_t kOffSlot = align256(kOffKey + 4 * (size_t)kNoAllocMaxParticles);   // u32[n]
constexpr size_t kOffTmp = align256(kOffSlot + 4 * (size_t)kNoAllocMaxParticles);   // u32[n]
constexpr size_t kOffTiles = align256(kOffTmp + 4 * (size_t)kNoAllocMaxParticles);  // u32[tiles]
constexpr size_t kMaxTiles = ((size_t)kNoAllocMaxCells + 1 + tsph::kScanTile - 1) / tsph::kScanTile;
constexpr size_t kOffBx = align256(kOffTiles + 4 * kMaxTiles);                      // i64[axis+1]
constexpr size_t kOffBy = align256(kOffBx + 8 * ((size_t)kNoAllocMaxAxis + 1));      // i64[axis+1]
constexpr size_t kOffEscaped = align256(kOffBy + 8 * ((size_t)kNoAllocMaxAxis + 1));  // u32
constexpr size_t kOffCrowded = kOffEscaped + 4;                                       // u32
constexpr size_t kScratchBytes = align256(kOffCrowded + 4);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void *g_addr[kNoAllocMaxDevices] = {};

// host staging of the tables (guarded by g_mu; the call waits for its copies)
long long g_hbx[kNoAllocMaxAxis + 1];
long long g_hby[kNoAllocMaxAxis + 1];

int fail(int code, const char *msg) {
    tsph::set_last_error(msg);
    return code;
}

// device address of the scratch array on the current device (set up once)
int scratch_address(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(TSPH_ERR_CUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(TSPH_ERR_UNSUPPORTED, "device index too large");
    if (!g_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return fail(TSPH_ERR_CUDA, cudaGetErrorString(e));
        g_addr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_addr[dev]);
    return TSPH_OK;
}

// cell and histogram slot of particle i; outside the grid: not binned
__global__ void k_na_bin(const double *__restrict__ r, int n, tsph::Grid g,
                         uint32_t *__restrict__ key, uint32_t *__restrict__ slot,
                         uint32_t *__restrict__ counts, uint32_t *__restrict__ escaped) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int cx, cy;
    const double2 ri = make_double2(r[2 * (size_t)i], r[2 * (size_t)i + 1]);
    const uint32_t k = tsph::cell_key(g, ri, 0xffffffffu, &cx, &cy);
    key[i] = k;
    if (k == (uint32_t)g.ncells) {
        atomicAdd(escaped, 1u);
        return;
    }
    slot[i] = atomicAdd(counts + k, 1u);
}

__global__ void k_na_place(const uint32_t *__restrict__ key, const uint32_t *__restrict__ slot,
                           int n, int ncells, const int32_t *__restrict__ start,
                           uint32_t *__restrict__ tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = key[i];
    if (k == (uint32_t)ncells) return;
    tmp[start[k] + slot[i]] = (uint32_t)i;
}

// final position: cell start + number of cell members with a smaller index
// (the reference appends in index order, so each cell list is ascending);
// cells above the occupancy bound are flagged and left unranked
__global__ void k_na_rank(const uint32_t *__restrict__ key, int n, int ncells,
                          const int32_t *__restrict__ start, const uint32_t *__restrict__ tmp,
                          int32_t *__restrict__ list, uint32_t *__restrict__ crowded) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = key[i];
    if (k == (uint32_t)ncells) return;
    const int lo = start[k], hi = start[k + 1];
    if (hi - lo > kNoAllocMaxPerCell) {
        *crowded = 1u;
        return;
    }
    int rank = 0;
    for (int m = lo; m < hi; m++) rank += tmp[m] < (uint32_t)i ? 1 : 0;
    list[lo + rank] = i;
}

}  // namespace

extern "C" {

int tsph_particle_to_cell_noalloc(const tsph_constants *c, const tsph_domain *d, int n,
                                  const double *r_dev, int32_t *cell_start_dev,
                                  int32_t *cell_list_dev, void *stream, int *n_binned) {
    if (!c || !d || n < 0 || (n > 0 && (!r_dev || !cell_list_dev)) || !cell_start_dev)
        return fail(TSPH_ERR_ARG, "null or negative argument");
    if ((reinterpret_cast<uintptr_t>(r_dev) & 7u) ||
        (reinterpret_cast<uintptr_t>(cell_start_dev) & 3u) ||
        (reinterpret_cast<uintptr_t>(cell_list_dev) & 3u))
        return fail(TSPH_ERR_ARG, "misaligned buffer (r_dev needs 8-byte, the cell arrays 4-byte alignment)");
    if (n > kNoAllocMaxParticles)
        return fail(TSPH_ERR_ARG, "too many particles for the allocation-free binning (max 1048576)");
    if (!(c->h > 0) || !(c->kap > 0) || !(d->x_m > d->x_0) || !(d->y_m > d->y_0))
        return fail(TSPH_ERR_ARG, "bad constants or domain");
    // Divide_To_Cells, src/SPH_find_pairs.h:5-42
    const double kh = c->kap * c->h;
    const double of = c->h * 0.273;
    const double qx = (d->x_m - d->x_0 + of) / kh, qy = (d->y_m - d->y_0 + of) / kh;
    if (!(qx < kNoAllocMaxAxis) || !(qy < kNoAllocMaxAxis))
        return fail(TSPH_ERR_ARG, "grid too large for the allocation-free binning (max 8192 cells per axis)");
    const int ncx = (int)qx + 1, ncy = (int)qy + 1;
    if ((long long)ncx * ncy > kNoAllocMaxCells)
        return fail(TSPH_ERR_ARG, "grid too large for the allocation-free binning (max 1048576 cells)");
    const int ncells = ncx * ncy;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    std::lock_guard<std::mutex> lock(g_mu);
    unsigned char *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    uint32_t *counts = reinterpret_cast<uint32_t *>(base + kOffCounts);
    uint32_t *key = reinterpret_cast<uint32_t *>(base + kOffKey);
    uint32_t *slot = reinterpret_cast<uint32_t *>(base + kOffSlot);
    uint32_t *tmp = reinterpret_cast<uint32_t *>(base + kOffTmp);
    uint32_t *tiles = reinterpret_cast<uint32_t *>(base + kOffTiles);
    long long *bx = reinterpret_cast<long long *>(base + kOffBx);
    long long *by = reinterpret_cast<long long *>(base + kOffBy);
    uint32_t *escaped = reinterpret_cast<uint32_t *>(base + kOffEscaped);
    uint32_t *crowded = reinterpret_cast<uint32_t *>(base + kOffCrowded);

    for (int k = 0; k <= ncx; k++) g_hbx[k] = tsph::cell_lower_bound(k, d->x_0, of, kh);
    for (int k = 0; k <= ncy; k++) g_hby[k] = tsph::cell_lower_bound(k, d->y_0, of, kh);

    // on an error after work was queued, wait for that work before returning
    // (and releasing the mutex), so the next call cannot overlap it on the array
#define NA_CK(call)                                                             \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) {                                                \
            cudaStreamSynchronize(st);                                          \
            return fail(TSPH_ERR_CUDA, cudaGetErrorString(e_));                 \
        }                                                                       \
    } while (0)
    NA_CK(cudaMemcpyAsync(bx, g_hbx, 8 * (size_t)(ncx + 1), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(by, g_hby, 8 * (size_t)(ncy + 1), cudaMemcpyHostToDevice, st));
    // what must start at zero: the histogram and the two flags
    NA_CK(cudaMemsetAsync(counts, 0, 4 * ((size_t)ncells + 1), st));
    NA_CK(cudaMemsetAsync(escaped, 0, 8, st));

    tsph::Grid g{};
    g.ax = tsph::Axis{bx, nullptr, ncx};
    g.ay = tsph::Axis{by, nullptr, ncy};
    g.ncx = ncx;
    g.ncy = ncy;
    g.ncells = ncells;
    g.khf = (float)kh;
    const int nb = n > 0 ? (n + tsph::kBlock - 1) / tsph::kBlock : 1;
    if (n > 0)
        k_na_bin<<<nb, tsph::kBlock, 0, st>>>(r_dev, n, g, key, slot, counts, escaped);
    const int ntiles = (ncells + 1 + tsph::kScanTile - 1) / tsph::kScanTile;
    uint32_t *start = reinterpret_cast<uint32_t *>(cell_start_dev);
    tsph::k_scan_tiles<<<ntiles, tsph::kScanThreads, 0, st>>>(counts, start, tiles, ncells);
    tsph::k_scan_sums<<<1, tsph::kScanThreads, 0, st>>>(tiles, ntiles, start, ncells);
    tsph::k_scan_add<<<(ncells + tsph::kBlock - 1) / tsph::kBlock, tsph::kBlock, 0, st>>>(start, tiles,
                                                                                       ncells);
    if (n > 0) {
        k_na_place<<<nb, tsph::kBlock, 0, st>>>(key, slot, n, ncells, cell_start_dev, tmp);
        k_na_rank<<<nb, tsph::kBlock, 0, st>>>(key, n, ncells, cell_start_dev, tmp, cell_list_dev,
                                               crowded);
    }
    NA_CK(cudaGetLastError());
    uint32_t flags[2] = {0u, 0u};  // escaped, crowded
    int32_t total = 0;
    NA_CK(cudaMemcpyAsync(flags, escaped, 8, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(&total, cell_start_dev + ncells, 4, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
#undef NA_CK
    if (n_binned) *n_binned = total;
    if (flags[1])
        return fail(TSPH_ERR_ARG, "a cell holds more than 4096 particles (max for the allocation-free binning)");
    if (flags[0]) return fail(TSPH_ERR_ESCAPED, "particles outside the cell grid were left out of the lists");
    return TSPH_OK;
}

}  // extern "C"
