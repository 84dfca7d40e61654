// tsph_kernels.cuh -- templated CUDA kernels of the WCSPH step.
//
// Instantiated twice: tsph_kernels_f32.cu (T = float: FP32 pair math, FP64
// positions) and tsph_kernels_f64.cu (T = double, compiled with -fmad=false so
// the arithmetic rounds like the reference's C++ on x86-64).
//
// Neighbour iteration everywhere follows the reference's cell order
// zz, zp, pp, pz, pm, zm, mm, mz, mp (src/SPH_interaction.h:26-36); inside a
// cell walls come before fluid and both are ascending by particle index, which
// is the reference's list order whenever walls are created first (every
// reference case does).  Cells that the reference reaches only by wrapping the
// column index (c+1 from the top row, c-1 from the bottom row, or a key outside
// [0, ncells)) are skipped: their particles are at least (ncy-2)*kh > 2h away,
// so their contribution in the reference is exactly zero (W = dW = 0 for
// q > 2, src/SPH_kernel.h:68-71).  The system rejects grids with ncy < 4.
#pragma once

#include "tsph_internal.cuh"

namespace tsph {

// ---------------------------------------------------------------- helpers
static __constant__ int kDX[9] = {0, 0, 1, 1, 1, 0, -1, -1, -1};
static __constant__ int kDY[9] = {0, 1, 1, 0, -1, -1, -1, 0, 1};

__device__ __forceinline__ int n_live(const uint32_t *fstart, int ncells) {
    return (int)__ldg(fstart + ncells);
}

// FP64 Wendland C2 kernel with the reference's float roundings,
// src/SPH_kernel.h:52-77.
__device__ __forceinline__ void wendland64(double r, double h, double awen, double bwen,
                                           double &W, double &F) {
    const double qq = r / h;
    const float wqq1 = 1.f - 0.5f * qq;
    const float wqq2 = wqq1 * wqq1;
    const float wqq = qq + qq + 1.f;
    if (qq <= 2.0) {
        W = awen * wqq * wqq2 * wqq2;
        F = bwen * qq * wqq2 * wqq1 / r;
    } else {
        W = 0.0;
        F = 0.0;
    }
    if (r == 0.0) {
        W = awen;
        F = 0.0;
    }
}

// FP32 Wendland C2: W and (dW/dr)/r for 0 < q <= 2 (caller tests the range).
__device__ __forceinline__ void wendland32(float r2, const Phys<float> &P, float &W, float &F,
                                           bool want_w) {
    const float r = r2 * rsqrtf(r2);
    const float q = r * P.inv_h;
    const float w1 = fmaf(-0.5f, q, 1.f);
    const float w2 = w1 * w1;
    F = P.bwen_h * w2 * w1;
    if (want_w) W = P.awen * fmaf(2.f, q, 1.f) * w2 * w2;
}

template <typename T> struct Acc {
    T ax, ay, cont, diff;
};

// One WCSPH pair (a = target, b = neighbour), FP64, reference arithmetic:
// momentum src/SPH_interaction.h:107-116, AV src/SPH_viscouse_forces.h:7-25,
// continuity + Fourtakas term src/SPH_interaction.h:118-128 and
// src/SPH_viscouse_forces.h:45-61.
__device__ __forceinline__ void pair64(double drx, double dry, double dvx, double dvy,
                                       double arho, double nrho, double ap, double np_,
                                       const Phys<double> &P, Acc<double> &acc) {
    const double drs = sqrt((drx * drx) + (dry * dry));
    const double qq = drs / P.h;
    if (!(qq <= 2.0) || drs == 0.0) return;  // W = dW = 0: exact zero contribution
    const double drdv = drx * dvx + dry * dvy;
    double W, F;
    wendland64(drs, P.h, P.awen, P.bwen, W, F);
    const double dWx = drx * F, dWy = dry * F;
    const double dvdW = dvx * dWx + dvy * dWy;
    const double drdW = drx * dWx + dry * dWy;
    const double p_temp = (ap + np_) / (arho * nrho);
    double visco = 0;
    {
        const double rbar = 0.5 * (arho + nrho);
        const double vmax = drdv > P.alpha ? drdv : P.alpha;
        if (drdv < 0) {
            const double mu = P.h * drdv / (drs * drs + 0.01 * P.h * P.h);
            visco = -vmax * P.c0 * mu / rbar;
        }
    }
    acc.ax -= dWx * (p_temp + visco) * P.m;
    acc.ay -= dWy * (p_temp + visco) * P.m;
    const double cb = P.c0 * P.c0 * P.rho0 / 7.;
    const double dpH = 1. + dry * P.rho0 * P.g / cb;
    const double drhoH = P.rho0 * pow(dpH, 1. / 7) - P.rho0;
    const double psi = 2. * P.c0 * P.h * P.delta * ((nrho - arho) - drhoH) /
                       (drs * drs + 0.01 * P.h * P.h);
    const double DT = psi * drdW * P.m / nrho;
    acc.cont += dvdW * P.m;
    acc.diff -= DT;
}

// The same pair in FP32 with the algebra rearranged for the FP32 pipe:
// dW = dr F, dv.dW = F dr.dv, dr.dW = r^2 F; AV and the delta-term share one
// reciprocal of (r^2 + eps h^2); rho0((1+x)^(1/7) - 1) by its series
// x/7 - 3x^2/49 (|x| = |7 g dy / c0^2| < 1e-3, series error < 1e-10 relative);
// densities enter as rho - rho0 where they are subtracted.  The constant m is
// applied once per particle by the caller.
__device__ __forceinline__ void pair32(float drx, float dry, float dvx, float dvy,
                                       float ra, float sa, float pa_ra, float ia,
                                       float rb, float sb, float pb, const Phys<float> &P,
                                       Acc<float> &acc) {
    const float r2 = fmaf(drx, drx, dry * dry);
    if (!(r2 <= P.four_h2) || r2 == 0.f) return;
    float W, F;
    wendland32(r2, P, W, F, false);
    const float drdv = fmaf(drx, dvx, dry * dvy);
    const float inv_den = __frcp_rn(r2 + P.eps_h2);
    const float ib = __frcp_rn(rb);
    // (pa + pb)/(ra rb) = pa/ra * (1/rb) + pb * (1/ra)(1/rb)
    float pterm = (pa_ra + pb * ia) * ib;
    if (drdv < 0.f) pterm += P.k_av * drdv * inv_den * __frcp_rn(ra + rb);
    const float coef = F * pterm;
    acc.ax = fmaf(-drx, coef, acc.ax);
    acc.ay = fmaf(-dry, coef, acc.ay);
    acc.cont = fmaf(F, drdv, acc.cont);
    const float x = dry * P.xg;
    const float drhoH = P.rho0 * x * fmaf(-3.f / 49.f, x, 1.f / 7.f);
    const float psi = P.k_psi * ((sb - sa) - drhoH) * inv_den;
    acc.diff = fmaf(psi * r2, F * ib, acc.diff);
}

// ------------------------------------------------------------- binning
// Cell of a position with a starting guess (the previous cell, or -1).
__device__ __forceinline__ uint32_t cell_key(const Grid &g, double2 r, uint32_t guess_key,
                                             int *cx_out, int *cy_out) {
    if (!is_finite_d(r.x) || !is_finite_d(r.y)) return (uint32_t)g.ncells;
    int gx = 0, gy = 0;
    if (guess_key < (uint32_t)g.ncells) {
        gx = (int)(guess_key / (uint32_t)g.ncy);
        gy = (int)(guess_key - (uint32_t)gx * (uint32_t)g.ncy);
    } else {
        gx = g.ncx >> 1;
        gy = g.ncy >> 1;
    }
    const int cx = axis_cell(g.ax, r.x, gx);
    const int cy = axis_cell(g.ay, r.y, gy);
    if (cx < 0 || cy < 0 || cx >= g.ncx || cy >= g.ncy) return (uint32_t)g.ncells;
    *cx_out = cx;
    *cy_out = cy;
    return (uint32_t)(cy + cx * g.ncy);
}

__device__ __forceinline__ float2 cell_local(const Grid &g, double2 r, int cx, int cy) {
    return make_float2((float)(r.x - __ldg(g.ax.org + cx)), (float)(r.y - __ldg(g.ay.org + cy)));
}

// The sort kernels take an optional gate: when `gate` is given and holds 0
// the kernel does nothing (a rebuild that a CUDA graph carries but that only
// runs when a device-side check asked for it).
__device__ __forceinline__ bool gated_off(const uint32_t *gate) {
    return gate != nullptr && __ldg(gate) == 0u;
}

// dead particles (removed) get the last bucket without a range check
static __global__ void k_bin_keep_dead(const double2 *__restrict__ r, const uint32_t *__restrict__ old_key,
                                const int *__restrict__ n_ptr, Grid g,
                                uint32_t *__restrict__ key, uint32_t *__restrict__ slot,
                                uint32_t *__restrict__ counts, uint32_t *__restrict__ health,
                                const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *n_ptr) return;
    uint32_t k;
    if (old_key[i] == (uint32_t)g.ncells) {
        k = (uint32_t)g.ncells;
    } else {
        int cx, cy;
        k = cell_key(g, r[i], old_key[i], &cx, &cy);
        if (k == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
    }
    key[i] = k;
    slot[i] = atomicAdd(counts + k, 1u);
}

// ------------------------------------------------------------- scan
// Exclusive scan of counts[0, n) into out[0, n] (out[n] = total), in three
// launches: per-block scan of 4096 items, scan of the block sums, add.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total) {
    __shared__ uint32_t warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t warp_off = wid ? warp_sums[wid - 1] : 0u;
    *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_off + x - v;
}

static __global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t *__restrict__ in,
                                                            uint32_t *__restrict__ out,
                                                            uint32_t *__restrict__ tile_sums, int n) {
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan(s, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// the same, and the histogram is left zeroed for its next use
static __global__ void __launch_bounds__(kScanThreads) k_scan_tiles_clear(uint32_t *__restrict__ in,
                                                                         uint32_t *__restrict__ out,
                                                                         uint32_t *__restrict__ tile_sums,
                                                                         int n,
                                                                         const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        if (base + k < n) in[base + k] = 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan(s, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

// add the tile offsets over chunks of blockDim.x items (grid-stride over
// the chunks, so any grid size gives the same result: a gated launch can
// use a small grid); each chunk sums the tile totals before its own tile
// (at most a few hundred), the last chunk writes the grand total to out[n]
static __global__ void k_scan_add_tiles(uint32_t *__restrict__ out,
                                        const uint32_t *__restrict__ tile_sums, int ntiles, int n,
                                        const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    __shared__ uint32_t red[kBlock / 32];
    const int nch = max(1, (n + (int)blockDim.x - 1) / (int)blockDim.x);
    for (int c = blockIdx.x; c < nch; c += gridDim.x) {
        const int i0 = c * blockDim.x;
        const int t = i0 / kScanTile;
        const bool last = c == nch - 1;
        const int upto = last ? ntiles : t;
        uint32_t acc = 0;
        for (int u = threadIdx.x; u < upto; u += blockDim.x) acc += tile_sums[u];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        uint32_t tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
        uint32_t off = tot;
        if (last) {
            // total of all tiles; the offset of this chunk's own tile excludes it
            if (threadIdx.x == 0) out[n] = tot;
            uint32_t mine = 0;
            if (t < ntiles) mine = tile_sums[t];
            uint32_t after = 0;
            for (int u = t + 1; u < ntiles; u++) after += tile_sums[u];
            off = tot - mine - after;
        }
        const int i = i0 + threadIdx.x;
        if (i < n) out[i] += off;
        __syncthreads();  // red is reused by the next chunk
    }
}

static __global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t *__restrict__ tile_sums, int ntiles,
                                                           uint32_t *__restrict__ out, int n) {
    // one block; ntiles <= kScanTile
    const int base = threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < ntiles) ? tile_sums[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t off = block_exclusive_scan(s, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < ntiles) tile_sums[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) out[n] = total;
}

static __global__ void k_scan_add(uint32_t *__restrict__ out, const uint32_t *__restrict__ tile_sums, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += tile_sums[i / kScanTile];
}

// ------------------------------------------------------ stable scatter
// place: provisional slot from the atomic histogram.  The order key inside a
// cell is the particle index (FP64 build: the reference's list order) or, when
// `r` is given, (y, index) (FP32 build: cells sorted by height, which lets the
// pair kernel stop early in the rows above and below).
static __global__ void k_place(const uint32_t *__restrict__ key, const uint32_t *__restrict__ slot,
                        const uint32_t *__restrict__ id, const int *__restrict__ n_ptr,
                        const uint32_t *__restrict__ start, uint32_t *__restrict__ tmp_id,
                        uint32_t *__restrict__ tmp_src, const double2 *__restrict__ r,
                        long long *__restrict__ tmp_y, const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    // grid-stride: any grid size (a gated launch can use a small grid)
    const int n = *n_ptr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t d = start[key[i]] + slot[i];
        tmp_id[d] = id[i];
        tmp_src[d] = (uint32_t)i;
        if (r) tmp_y[d] = ordered_bits(r[i].y);
    }
}

// rank: final position = cell start + number of cell members that order
// before this one (the order key inside a cell as in k_place); then move
// the particle's record straight to its final
// slot: D[final] = src[s], recomputing loc; optional acceleration, density
// rate, pressure and old state travel along
template <typename T>
__global__ void k_rank_scatter(const uint32_t *__restrict__ key, const int *__restrict__ n_ptr,
                               const uint32_t *__restrict__ start, const uint32_t *__restrict__ tmp_id,
                               const uint32_t *__restrict__ tmp_src, const long long *__restrict__ tmp_y,
                               Grid g, const double2 *__restrict__ sr,
                               const typename V2<T>::t *__restrict__ sv, const T *__restrict__ srho,
                               const uint32_t *__restrict__ sid,
                               const typename V2<T>::t *__restrict__ sa, const T *__restrict__ sdrho,
                               const T *__restrict__ sp, FluidState<T> D,
                               const double2 *__restrict__ or2, const typename V2<T>::t *__restrict__ ov2,
                               const T *__restrict__ orho2, OldState<T> O,
                               const uint32_t *__restrict__ gate,
                               const uint8_t *__restrict__ stype, float2 *__restrict__ lbin,
                               uint32_t *__restrict__ gen, uint32_t *__restrict__ runs) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == 0) {
        if (gen) atomicAdd(gen, 1u);    // a new order: neighbour lists built before are stale
        if (runs) atomicAdd(runs, 1u);  // executions of a conditional sort
    }
    if (j >= *n_ptr) return;
    const uint32_t src = tmp_src[j];
    const uint32_t k = key[src];
    uint32_t f = (uint32_t)j;
    if (k != (uint32_t)g.ncells) {
        const uint32_t lo = start[k], hi = start[k + 1];
        const uint32_t me = tmp_id[j];
        uint32_t rank = 0;
        if (tmp_y) {
            const long long my = tmp_y[j];
            for (uint32_t m = lo; m < hi; m++) {
                const long long ym = tmp_y[m];
                rank += (ym < my || (ym == my && tmp_id[m] < me)) ? 1u : 0u;
            }
        } else {
            for (uint32_t m = lo; m < hi; m++) rank += (tmp_id[m] < me) ? 1u : 0u;
        }
        f = lo + rank;
    }
    const double2 r = sr[src];
    D.r[f] = r;
    D.v[f] = sv[src];
    D.rho[f] = srho[src];
    D.id[f] = sid[src];
    D.key[f] = k;
    float2 l = make_float2(0.f, 0.f);
    if (k < (uint32_t)g.ncells) {
        const int cx = (int)(k / (uint32_t)g.ncy);
        const int cy = (int)k - cx * g.ncy;
        l = cell_local(g, r, cx, cy);
    }
    D.loc[f] = l;
    if (lbin) lbin[f] = l;
    if (sa) D.a[f] = sa[src];
    if (sdrho) D.drho[f] = sdrho[src];
    if (sp) D.p[f] = sp[src];
    if (stype) D.type[f] = stype[src];
    if (or2) {
        O.r[f] = or2[src];
        O.v[f] = ov2[src];
        O.rho[f] = orho2[src];
    }
}

// ------------------------------------------------------------- EOS
template <typename T>
__global__ void k_eos(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                      WallState<T> Wl, int nw, Phys<T> P, uint32_t *__restrict__ health) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    T s;
    T *pout;
    if (i < nw) {
        s = Wl.rho[i];
        pout = Wl.p + i;
    } else {
        const int f = i - nw;
        if (f >= n_live(fstart, ncells)) return;
        s = F.rho[f];
        pout = F.p + f;
    }
    const T full = rho_full(s, P.rho0);
    if (!(full >= T(0) && full <= T(1500))) atomicOr(health, full == full ? kHealthDensity : kHealthNan);
    *pout = eos(s, P);
}

// -------------------------------------------------------- integrators
// Integrate_SymplecticPredictor, src/SPH_integration.h:266-287 (in place;
// saves the old state).  Walls: rho_o = rho, rho += drho dt/2, r and v fixed.
template <typename T>
__global__ void k_predict_inplace(FluidState<T> F, OldState<T> O, const uint32_t *__restrict__ fstart,
                                  int ncells, WallState<T> Wl, int nw, T dt) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        const T r = Wl.rho[i];
        Wl.rho_o[i] = r;
        if constexpr (std::is_same<T, float>::value) Wl.rho[i] = r + Wl.drho[i] * dt * 0.5f;
        else Wl.rho[i] = r + Wl.drho[i] * dt * 0.5;
        return;
    }
    const int f = i - nw;
    if (f >= n_live(fstart, ncells)) return;
    const double2 r = F.r[f];
    const auto v = F.v[f];
    const auto a = F.a[f];
    const T rho = F.rho[f];
    O.r[f] = r;
    O.v[f] = v;
    O.rho[f] = rho;
    F.rho[f] = rho + F.drho[f] * dt * T(0.5);
    F.r[f] = make_double2(r.x + (double)v.x * (double)dt * 0.5, r.y + (double)v.y * (double)dt * 0.5);
    typename V2<T>::t nv;
    nv.x = v.x + a.x * dt * T(0.5);
    nv.y = v.y + a.y * dt * T(0.5);
    F.v[f] = nv;
}

// rho = rho_o (2 - eps)/(2 + eps), eps = -(drho/rho) dt (src/SPH_integration.h:298-299),
// on stored densities
template <typename T> __device__ __forceinline__ T corrector_rho(T rho_o_s, T rho_s, T drho, T dt, T rho0) {
    if constexpr (std::is_same<T, float>::value) {
        const float rho = rho0 + rho_s;
        const float e = (-drho / rho) * dt;
        const float inv = 1.f / (2.f + e);
        // (rho0 + s_o)(2-e)/(2+e) - rho0 = s_o (2-e)/(2+e) - rho0 * 2e/(2+e)
        return rho_o_s * ((2.f - e) * inv) - rho0 * (2.f * e * inv);
    } else {
        const double epsilon = (-drho / rho_s) * dt;
        return rho_o_s * ((2. - epsilon) / (2. + epsilon));
    }
}

// Integrate_SymplecticCorrector, src/SPH_integration.h:289-309 (in place)
template <typename T>
__global__ void k_correct_inplace(FluidState<T> F, OldState<T> O, const uint32_t *__restrict__ fstart,
                                  int ncells, WallState<T> Wl, int nw, T dt, T rho0) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        Wl.rho[i] = corrector_rho(Wl.rho_o[i], Wl.rho[i], Wl.drho[i], dt, rho0);
        return;
    }
    const int f = i - nw;
    if (f >= n_live(fstart, ncells)) return;
    F.rho[f] = corrector_rho(O.rho[f], F.rho[f], F.drho[f], dt, rho0);
    const auto vo = O.v[f];
    const auto a = F.a[f];
    typename V2<T>::t nv;
    nv.x = vo.x + a.x * dt;
    nv.y = vo.y + a.y * dt;
    F.v[f] = nv;
    const double2 ro = O.r[f];
    F.r[f] = make_double2(ro.x + ((double)nv.x + (double)vo.x) * (double)dt * 0.5,
                          ro.y + ((double)nv.y + (double)vo.y) * (double)dt * 0.5);
}

// RemoveParticlesOutOfDomain, src/SPH_btdebug.h:4-31: fluid outside
// [x0-eps, xm-eps] x [y0-eps, ym+eps] (eps = 0.01) is marked removed (key =
// ncells) and dropped by the next binning.
__device__ __forceinline__ bool out_of_domain(double2 r, Box box) {
    return (r.y < (box.y0 - 0.01)) || (r.y > box.ym + 0.01) || (r.x < box.x0 - 0.01) ||
           (r.x > box.xm - 0.01);
}

// ---------------------------------------------------------- pair loop
// MODE_LISTS (pair kernel over pair records only): build and store the
// neighbour lists, compute nothing else
enum { MODE_FORCES = 0, MODE_CORRECT = 1, MODE_DIGEST = 2, MODE_LISTS = 3 };

// 1/x by the hardware's approximate reciprocal (rcp.approx.ftz.f32)
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// One set of pair records (fluid rows or walls; FP32 pair kernel over pair
// records): per row, t = (x, row kh + y) and y = (y, row) with (x, y) the
// position relative to the row's cell, v = (vx, vy, rho - rho0, p / rho),
// inv = 1 / rho.  Written by whichever kernel last changed the row (the
// predictor, the corrector, the walls' density kernels) or by k_pair_records.
struct PairRec {
    float4 *e;  // {x - x of the particle's own cell, y - y of that cell, cell row, 1/rho}
    float4 *v;  // {vx, vy, rho - rho0, p/rho}
};

// a wall's density-dependent record fields (walls do not move: the position
// part of e stays as k_pair_records wrote it)
__device__ __forceinline__ void wall_record(const PairRec &RW, int w, float s,
                                            const Phys<float> &P) {
    const float ib = rcp_approx(P.rho0 + s);
    RW.v[w] = make_float4(0.f, 0.f, s, eos(s, P) * ib);
    reinterpret_cast<float *>(RW.e + w)[3] = ib;
}

// RemoveParticlesOutOfDomain inside the fused step (src/SPH_btdebug.h:4-31).
// The reference erases inside a forward loop, so the particle right after an
// erased one is not examined in that call.  The corrector lists the fluid it
// moved outside the box as erase candidates (their cell kept aside, no
// histogram slot yet); k_resolve_removal then erases a candidate unless the
// run of candidates just before it (in index order, over present indices)
// has odd length, and counts every listed row into the histogram.
struct Removal {
    uint8_t *cand = nullptr;  // [particle index]: erase candidate this step
    uint32_t *list = nullptr; // rows of the candidates
    uint32_t *count = nullptr;
    int cap = 0;
    const uint32_t *ids = nullptr;  // particle index of each row of the corrected state
};
constexpr int kRemovalCap = 8192;  // candidates resolved per step

struct PairOut {  // where MODE_CORRECT writes the new (unsorted) state
    double2 *r;
    void *v;
    void *rho;
    uint32_t *key, *slot, *counts;
    Box box;
    BoxBits boxb;
    Removal rm{};
};

// a listed erase candidate: its cell if it survives the erase, no slot yet;
// false when the list is full (the candidate is then erased at once)
__device__ __forceinline__ bool list_removal(const Removal &rm, int row) {
    if (!rm.list) return false;
    const uint32_t k = atomicAdd(rm.count, 1u);
    if (k >= (uint32_t)rm.cap) return false;
    rm.list[k] = (uint32_t)row;
    rm.cand[rm.ids[row]] = 1;
    return true;
}

// ordered bits with -0.0 folded onto +0.0 (they compare equal in FP64)
__host__ __device__ inline long long ordered_bits_fold0(double x) {
    const long long o = ordered_bits(x);
    return o == -1LL ? 0LL : o;
}

inline BoxBits make_box_bits(const Box &b) {
    return BoxBits{ordered_bits_fold0(b.x0 - 0.01), ordered_bits_fold0(b.xm - 0.01),
                   ordered_bits_fold0(b.y0 - 0.01), ordered_bits_fold0(b.ym + 0.01)};
}

// in-support test: 0 < r2 <= (2h)^2 as one unsigned compare of the bits
__device__ __forceinline__ uint32_t in_support(float r2, uint32_t four_h2_bits) {
    return (uint32_t)(__float_as_uint(r2) - 1u) < four_h2_bits ? 1u : 0u;
}

// Phase-1 scans of one staged row range (lists of the tiled pair kernels,
// entries STRIDE apart): every in-support candidate
// (r^2 <= 4h^2) appends its entry (staged index << 2 | row code).  The entry
// is written unconditionally and kept by advancing the list pointer.  Only
// the particle's own cell can hold a coincident particle or the particle
// itself; there (EXCL) the test is 0 < r^2 <= 4h^2, as one unsigned compare
// of the bits, elsewhere a plain float compare.  Rows are sorted by y, so
// the row above is walked upwards and the row below downwards until |dy|
// passes `reach`, two candidates per iteration (the test of the second ends
// the walk; a candidate beyond the reach fails the support test anyway).
template <bool EXCL> __device__ __forceinline__ bool support_test(float r2, float h2) {
    if constexpr (EXCL) return in_support(r2, __float_as_uint(h2)) != 0u;
    else return r2 <= h2;
}

template <int STRIDE, bool EXCL>
__device__ __forceinline__ uint16_t *scan_own(const float2 *__restrict__ loc, int j0, int j1,
                                              float bx, float by, float h2, uint16_t *w) {
    uint32_t ent = ((uint32_t)j0 << 2) | 1u;
    int j = j0;
    for (; j + 1 < j1; j += 2, ent += 8u) {
        const float2 l0 = loc[j], l1 = loc[j + 1];
        const float dx0 = bx - l0.x, dy0 = by - l0.y;
        const float dx1 = bx - l1.x, dy1 = by - l1.y;
        const bool in0 = support_test<EXCL>(fmaf(dx0, dx0, dy0 * dy0), h2);
        const bool in1 = support_test<EXCL>(fmaf(dx1, dx1, dy1 * dy1), h2);
        *w = (uint16_t)ent;
        w += in0 ? STRIDE : 0;
        *w = (uint16_t)(ent + 4u);
        w += in1 ? STRIDE : 0;
    }
    if (j < j1) {
        const float2 l = loc[j];
        const float dx = bx - l.x, dy = by - l.y;
        *w = (uint16_t)ent;
        w += support_test<EXCL>(fmaf(dx, dx, dy * dy), h2) ? STRIDE : 0;
    }
    return w;
}

template <int STRIDE>
__device__ __forceinline__ uint16_t *scan_above(const float2 *__restrict__ loc, int j0, int j1,
                                                float bx, float by, float h2, float reach,
                                                uint16_t *w) {
    uint32_t ent = ((uint32_t)j0 << 2) | 2u;
    int j = j0;
    bool go = true;
    for (; go && j + 1 < j1; j += 2, ent += 8u) {
        const float2 l0 = loc[j], l1 = loc[j + 1];
        const float dx0 = bx - l0.x, dy0 = by - l0.y;
        const float dx1 = bx - l1.x, dy1 = by - l1.y;
        const bool in0 = fmaf(dx0, dx0, dy0 * dy0) <= h2;
        const bool in1 = fmaf(dx1, dx1, dy1 * dy1) <= h2;
        *w = (uint16_t)ent;
        w += in0 ? STRIDE : 0;
        *w = (uint16_t)(ent + 4u);
        w += in1 ? STRIDE : 0;
        go = dy1 >= -reach;
    }
    if (go && j < j1) {
        const float2 l = loc[j];
        const float dx = bx - l.x, dy = by - l.y;
        *w = (uint16_t)ent;
        w += fmaf(dx, dx, dy * dy) <= h2 ? STRIDE : 0;
    }
    return w;
}

template <int STRIDE>
__device__ __forceinline__ uint16_t *scan_below(const float2 *__restrict__ loc, int j0, int j1,
                                                float bx, float by, float h2, float reach,
                                                uint16_t *w) {
    uint32_t ent = ((uint32_t)(j1 - 1) << 2);
    int j = j1 - 1;
    bool go = true;
    for (; go && j - 1 >= j0; j -= 2, ent -= 8u) {
        const float2 l0 = loc[j], l1 = loc[j - 1];
        const float dx0 = bx - l0.x, dy0 = by - l0.y;
        const float dx1 = bx - l1.x, dy1 = by - l1.y;
        const bool in0 = fmaf(dx0, dx0, dy0 * dy0) <= h2;
        const bool in1 = fmaf(dx1, dx1, dy1 * dy1) <= h2;
        *w = (uint16_t)ent;
        w += in0 ? STRIDE : 0;
        *w = (uint16_t)(ent - 4u);
        w += in1 ? STRIDE : 0;
        go = dy1 <= reach;
    }
    if (go && j >= j0) {
        const float2 l = loc[j];
        const float dx = bx - l.x, dy = by - l.y;
        *w = (uint16_t)ent;
        w += fmaf(dx, dx, dy * dy) <= h2 ? STRIDE : 0;
    }
    return w;
}

// RemoveParticlesOutOfDomain's test (src/SPH_btdebug.h:16-19) on the ordered
// bits of the coordinates against precomputed ordered thresholds: integer
// compares instead of FP64 ones (GB300 issues FP64 at a small fraction of the
// FP32 rate).  NaN coordinates compare false, as in FP64.
__device__ __forceinline__ bool out_of_domain_bits(double2 r, const BoxBits &b) {
    const long long ox = ordered_bits_fold0(r.x), oy = ordered_bits_fold0(r.y);
    const long long ax = __double_as_longlong(r.x) & 0x7fffffffffffffffLL;
    const long long ay = __double_as_longlong(r.y) & 0x7fffffffffffffffLL;
    const bool nan = ax > 0x7ff0000000000000LL || ay > 0x7ff0000000000000LL;
    return !nan && (oy < b.y_lo || oy > b.y_hi || ox < b.x_lo || ox > b.x_hi);
}

template <typename T> struct Nbr {  // neighbour fields read by the pair loop
    const double2 *r;
    const float2 *loc;
    const typename V2<T>::t *v;
    const T *rho;
    const T *p;                   // nullptr: compute EOS from rho
    const double2 *n = nullptr;   // wall normals (boundary-integral walls)
    const uint8_t *type = nullptr;  // row types (buffer zones): non-fluid rows are skipped
                                    // where the reference takes fluid neighbours only
};

template <typename T> struct BtAcc {
    T ax, ay, cont, diff, gamma;
};

// One pair of the boundary-integral flavour, src/SPH_interactionBT.h:99-172
// (a = fluid target, b = neighbour): a fluid neighbour adds the WCSPH terms
// and W m / rho_b to the Shepard sum gamma (a buffer-zone neighbour, `shep`
// false, adds the terms but not to gamma: the sum takes fluid-typed
// particles only); a wall neighbour with normal n_b
// adds W (p_temp + visco) dp n_b rho_b to the momentum sum and
// -(dv . n_b) W rho_b dp to the continuity sum (its diffusion term is not
// used).  Arithmetic in the reference's order; out-of-support pairs add
// exactly zero (W = dW = 0) and are skipped; at r = 0 the kernel value is
// awen, as in src/SPH_kernel.h:68-75.
template <typename T>
__device__ __forceinline__ void bt_pair(T drx, T dry, T dvx, T dvy, T arho, T nrho, T ap, T np_,
                                        bool wall, T nbx, T nby, const Phys<T> &P,
                                        BtAcc<T> &acc, bool shep = true) {
    T drs, W, F;
    if constexpr (std::is_same<T, double>::value) {
        drs = sqrt((drx * drx) + (dry * dry));
        if (!(drs / P.h <= 2.0)) return;
        wendland64(drs, P.h, P.awen, P.bwen, W, F);
    } else {
        const float r2 = fmaf(drx, drx, dry * dry);
        if (!(r2 <= P.four_h2)) return;
        if (r2 == 0.f) {
            drs = 0.f;
            W = P.awen;
            F = 0.f;
        } else {
            drs = sqrtf(r2);
            wendland32(r2, P, W, F, true);
        }
    }
    const T drdv = drx * dvx + dry * dvy;
    const T p_temp = (ap + np_) / (arho * nrho);
    T visco = 0;
    {
        const T rbar = T(0.5) * (arho + nrho);
        const T vmax = drdv > P.alpha ? drdv : P.alpha;
        if (drdv < 0) {
            const T mu = P.h * drdv / (drs * drs + T(0.01) * P.h * P.h);
            visco = -vmax * P.c0 * mu / rbar;
        }
    }
    if (wall) {
        acc.ax += W * (p_temp + visco) * P.dp * nbx * nrho;
        acc.ay += W * (p_temp + visco) * P.dp * nby * nrho;
        const T dvnb = dvx * nbx + dvy * nby;
        acc.cont -= dvnb * W * nrho * P.dp;
    } else {
        const T dWx = drx * F, dWy = dry * F;
        const T dvdW = dvx * dWx + dvy * dWy;
        const T drdW = drx * dWx + dry * dWy;
        acc.ax -= dWx * (p_temp + visco) * P.m;
        acc.ay -= dWy * (p_temp + visco) * P.m;
        T drhoH;
        if constexpr (std::is_same<T, double>::value) {
            const double cb = P.c0 * P.c0 * P.rho0 / 7.;
            const double dpH = 1. + dry * P.rho0 * P.g / cb;
            drhoH = P.rho0 * pow(dpH, 1. / 7) - P.rho0;
        } else {
            const float x = dry * P.xg;  // rho0((1+x)^(1/7) - 1) by its series, as pair32
            drhoH = P.rho0 * x * fmaf(-3.f / 49.f, x, 1.f / 7.f);
        }
        const T psi = T(2) * P.c0 * P.h * P.delta * ((nrho - arho) - drhoH) /
                      (drs * drs + T(0.01) * P.h * P.h);
        const T DT = psi * drdW * P.m / nrho;
        acc.cont += dvdW * P.m;
        acc.diff -= DT;
        if (shep) acc.gamma += W * P.m / nrho;
    }
}

// Fluid rows: Compute_Forces (src/SPH_interaction.h:57-137 / SPH_interactionDBC.h:57-142)
// for every live fluid particle of the sorted state F, one thread per particle.
// MODE_CORRECT then applies the symplectic corrector (src/SPH_integration.h:
// 289-309) with the old state O and bins the new position (key + histogram
// slot), marking particles outside the domain as removed (src/SPH_btdebug.h:22).
template <typename T, int MODE, bool BT = false>
__global__ void __launch_bounds__(kBlock)
k_fluid_pairs(FluidState<T> F, const uint32_t *__restrict__ fstart,
              const uint32_t *__restrict__ wstart, Nbr<T> NF, Nbr<T> NW, Grid g, Phys<T> P,
              OldState<T> O, T dt, PairOut out, uint32_t *__restrict__ health,
              int32_t *__restrict__ dig_count, long long *__restrict__ dig_sum,
              int32_t *__restrict__ dig_xor, const uint32_t *__restrict__ wid) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncells = g.ncells;
    if (i >= n_live(fstart, ncells)) return;
    // buffer particles are neighbours but not targets (src/SPH_interaction.h:64)
    if (MODE == MODE_FORCES && F.type && F.type[i] != 0) return;
    const uint32_t key = F.key[i];
    const int cx = (int)(key / (uint32_t)g.ncy);
    const int cy = (int)key - cx * g.ncy;
    const double2 ra = F.r[i];
    const auto va = F.v[i];
    const T sa = F.rho[i];
    const T rho_a = rho_full(sa, P.rho0);
    const T pa = NF.p ? NF.p[i] : eos(sa, P);
    Acc<T> acc = {T(0), T(0), T(0), T(0)};
    BtAcc<T> bacc = {T(0), T(0), T(0), T(0), T(0)};
    int dcount = 0;
    long long dsum = 0;
    int dxor = 0;
    float2 la;
    float ia = 0.f, pa_ra = 0.f;
    if constexpr (std::is_same<T, float>::value) {
        la = F.loc[i];
        ia = __frcp_rn(rho_a);
        pa_ra = pa * ia;
    }
    for (int k = 0; k < 9; k++) {
        const int nx = cx + kDX[k], ny = cy + kDY[k];
        if (nx < 0 || ny < 0 || nx >= g.ncx || ny >= g.ncy) continue;
        const int c = ny + nx * g.ncy;
        const float offx = (float)(-kDX[k]) * g.khf;
        const float offy = (float)(-kDY[k]) * g.khf;
#pragma unroll 1
        for (int part = 0; part < 2; part++) {  // walls first, then fluid
            if constexpr (BT && MODE != MODE_DIGEST) {
                const Nbr<T> &N = part == 0 ? NW : NF;
                const uint32_t *st = part == 0 ? wstart : fstart;
                const int j0 = (int)__ldg(st + c), j1 = (int)__ldg(st + c + 1);
                for (int j = j0; j < j1; j++) {
                    if (part == 1 && j == i) continue;
                    T drx, dry;
                    if constexpr (std::is_same<T, float>::value) {
                        const float2 lb = __ldg(N.loc + j);
                        drx = (la.x - lb.x) + offx;
                        dry = (la.y - lb.y) + offy;
                    } else {
                        const double2 rb = __ldg(N.r + j);
                        drx = ra.x - rb.x;
                        dry = ra.y - rb.y;
                    }
                    const auto vb = __ldg(N.v + j);
                    const T nrho = rho_full(__ldg(N.rho + j), P.rho0);
                    const T pb = N.p ? __ldg(N.p + j) : eos(__ldg(N.rho + j), P);
                    T nbx = T(0), nby = T(0);
                    if (part == 0) {
                        const double2 nb = __ldg(N.n + j);
                        nbx = (T)nb.x;
                        nby = (T)nb.y;
                    }
                    const bool shep = part == 1 && !(N.type && __ldg(N.type + j) != 0);
                    bt_pair<T>(drx, dry, va.x - vb.x, va.y - vb.y, rho_a, nrho, pa, pb, part == 0,
                               nbx, nby, P, bacc, shep);
                }
                continue;
            }
            const Nbr<T> &N = part == 0 ? NW : NF;
            const uint32_t *st = part == 0 ? wstart : fstart;
            const int j0 = (int)__ldg(st + c), j1 = (int)__ldg(st + c + 1);
            for (int j = j0; j < j1; j++) {
                if (part == 1 && j == i) continue;
                if constexpr (MODE == MODE_DIGEST) {
                    // the reference's support test in FP64 with no FMA
                    // contraction: r/h <= 2, r = sqrt(dx*dx + dy*dy)
                    const double2 rb = __ldg(N.r + j);
                    const double drx = __dsub_rn(ra.x, rb.x), dry = __dsub_rn(ra.y, rb.y);
                    const double drs = __dsqrt_rn(__dadd_rn(__dmul_rn(drx, drx), __dmul_rn(dry, dry)));
                    if (__ddiv_rn(drs, P.hd) <= 2.0) {
                        const int nid = part == 0 ? (int)wid[j] : (int)F.id[j];
                        dcount++;
                        dsum += nid;
                        dxor ^= nid;
                    }
                } else if constexpr (std::is_same<T, float>::value) {
                    const float2 lb = __ldg(N.loc + j);
                    const float drx = (la.x - lb.x) + offx;
                    const float dry = (la.y - lb.y) + offy;
                    const float2 vb = __ldg(N.v + j);
                    const float sb = __ldg(N.rho + j);
                    const float rb = P.rho0 + sb;
                    const float pb = N.p ? __ldg(N.p + j) : eos(sb, P);
                    pair32(drx, dry, va.x - vb.x, va.y - vb.y, rho_a, sa, pa_ra, ia, rb, sb, pb,
                           P, acc);
                } else {
                    const double2 rb = __ldg(N.r + j);
                    const double2 vb = __ldg(N.v + j);
                    const double nrho = __ldg(N.rho + j);
                    const double pb = N.p ? __ldg(N.p + j) : eos(nrho, P);
                    pair64(ra.x - rb.x, ra.y - rb.y, va.x - vb.x, va.y - vb.y, rho_a, nrho, pa,
                           pb, P, acc);
                }
            }
        }
    }
    if constexpr (MODE == MODE_DIGEST) {
        dig_count[i] = dcount;
        dig_sum[i] = dsum;
        dig_xor[i] = dxor;
        return;
    } else {
        T ax, ay, drho;
        if constexpr (BT) {  // src/SPH_interactionBT.h:172-187 (eps = 0.01, src/SPH_defs.h:69)
            if (bacc.gamma > T(0.01)) {
                ax = bacc.ax / bacc.gamma - T(0);
                ay = bacc.ay / bacc.gamma - P.g;
                drho = bacc.cont / bacc.gamma + bacc.diff / bacc.gamma;
            } else {
                ax = T(0) - T(0);
                ay = T(0) - P.g;
                drho = T(0);
            }
        } else if constexpr (std::is_same<T, float>::value) {
            ax = acc.ax * P.m;
            ay = acc.ay * P.m - P.g;
            drho = (acc.cont - acc.diff) * P.m;
        } else {
            ax = acc.ax - 0.;
            ay = acc.ay - P.g;
            drho = acc.cont + acc.diff;
        }
        if constexpr (MODE == MODE_FORCES) {
            typename V2<T>::t a;
            a.x = ax;
            a.y = ay;
            F.a[i] = a;
            F.drho[i] = drho;
        } else {  // MODE_CORRECT: symplectic corrector into the output buffers
            const T so = O.rho[i];
            const T s_new = corrector_rho(so, sa, drho, dt, P.rho0);
            const auto vo = O.v[i];
            typename V2<T>::t nv;
            nv.x = vo.x + ax * dt;
            nv.y = vo.y + ay * dt;
            const double2 ro = O.r[i];
            const double2 rn =
                make_double2(ro.x + ((double)nv.x + (double)vo.x) * (double)dt * 0.5,
                             ro.y + ((double)nv.y + (double)vo.y) * (double)dt * 0.5);
            out.r[i] = rn;
            reinterpret_cast<typename V2<T>::t *>(out.v)[i] = nv;
            reinterpret_cast<T *>(out.rho)[i] = s_new;
            uint32_t nk;
            bool listed = false;
            int ncx_, ncy_;
            if (out_of_domain(rn, out.box)) {
                nk = cell_key(g, rn, key, &ncx_, &ncy_);  // kept if the erase skips it
                listed = list_removal(out.rm, i);
                if (!listed) {
                    nk = (uint32_t)ncells;
                    atomicOr(health, kHealthRemoved);
                }
            } else {
                nk = cell_key(g, rn, key, &ncx_, &ncy_);
                if (nk == (uint32_t)ncells) atomicOr(health, kHealthEscaped);
            }
            if (!(nv.x == nv.x) || !(nv.y == nv.y) || !(s_new == s_new)) atomicOr(health, kHealthNan);
            out.key[i] = nk;
            if (!listed) out.slot[i] = atomicAdd(out.counts + nk, 1u);
        }
    }
}

// BT_compute_density_BTGeo, src/SPH_BT.h:9-50, with
// Kernel_density_approximation_BT_update, src/SPH_kernel_approx.h:1838-1953:
// a wall particle's density is the Shepard density of the fluid in the 3x3
// cell block of its own cell, sum m W / sum m W / rho_b (1000 when the sum
// is 0), raised to at least 1000.  One thread per wall particle.
template <typename T>
__global__ void __launch_bounds__(kBlock)
k_bt_density(WallState<T> Wl, int nw, const uint32_t *__restrict__ fstart, Nbr<T> NF, Grid g,
             Phys<T> P) {
    pdl_enter();
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    const uint32_t key = Wl.key[w];
    const int cx = (int)(key / (uint32_t)g.ncy);
    const int cy = (int)key - cx * g.ncy;
    const double2 ra = Wl.r[w];
    float2 la = make_float2(0.f, 0.f);
    if constexpr (std::is_same<T, float>::value) la = Wl.loc[w];
    T Wsum = T(0), rhoWsum = T(0);
    for (int k = 0; k < 9; k++) {
        const int nx = cx + kDX[k], ny = cy + kDY[k];
        if (nx < 0 || ny < 0 || nx >= g.ncx || ny >= g.ncy) continue;
        const int c = ny + nx * g.ncy;
        const float offx = (float)(-kDX[k]) * g.khf;
        const float offy = (float)(-kDY[k]) * g.khf;
        const int j0 = (int)__ldg(fstart + c), j1 = (int)__ldg(fstart + c + 1);
        for (int j = j0; j < j1; j++) {
            if (NF.type && __ldg(NF.type + j) != 0) continue;  // fluid only (buffer zones)
            T W;
            if constexpr (std::is_same<T, float>::value) {
                const float2 lb = __ldg(NF.loc + j);
                const float drx = (la.x - lb.x) + offx, dry = (la.y - lb.y) + offy;
                const float r2 = fmaf(drx, drx, dry * dry);
                if (!(r2 <= P.four_h2)) continue;
                float F;
                if (r2 == 0.f) W = P.awen;
                else wendland32(r2, P, W, F, true);
            } else {
                const double2 rb = __ldg(NF.r + j);
                const double dx = ra.x - rb.x, dy = ra.y - rb.y;
                double F;
                wendland64(sqrt(dx * dx + dy * dy), P.h, P.awen, P.bwen, W, F);
            }
            const T nrho = rho_full(__ldg(NF.rho + j), P.rho0);
            Wsum += W * P.m / nrho;
            rhoWsum += P.m * W;
        }
    }
    T dens = Wsum > T(0) ? rhoWsum / Wsum : T(1000);
    if (dens < T(1000)) dens = T(1000);
    Wl.rho[w] = rho_stored_from_full<T>((double)dens, (double)P.rho0);
}

// Wall rows of the DBC flavour (src/SPH_interactionDBC.h:57-142): a = 0, drho
// from fluid neighbours (wall-wall pairs skipped, :84).  With `correct` the
// wall density is then advanced by the corrector (the mDBC flavour calls this
// with dbc = false: no pair loop, drho unchanged).
template <typename T>
__global__ void __launch_bounds__(kBlock)
k_wall_rows(WallState<T> Wl, int nw, const uint32_t *__restrict__ fstart, Nbr<T> NF, Grid g,
            Phys<T> P, bool dbc, bool correct, T dt, int32_t *__restrict__ dig_count,
            long long *__restrict__ dig_sum, int32_t *__restrict__ dig_xor,
            const uint32_t *__restrict__ fid, bool digest, PairRec RW) {
    pdl_enter();
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nw) return;
    T drho = Wl.drho[w];
    const T sa = Wl.rho[w];
    if (dbc || digest) {
        const uint32_t key = Wl.key[w];
        const int cx = (int)(key / (uint32_t)g.ncy);
        const int cy = (int)key - cx * g.ncy;
        const double2 ra = Wl.r[w];
        const T rho_a = rho_full(sa, P.rho0);
        const T pa = NF.p ? Wl.p[w] : eos(sa, P);
        Acc<T> acc = {T(0), T(0), T(0), T(0)};
        int dcount = 0;
        long long dsum = 0;
        int dxor = 0;
        float2 la;
        float ia = 0.f, pa_ra = 0.f;
        if constexpr (std::is_same<T, float>::value) {
            la = Wl.loc[w];
            ia = __frcp_rn(rho_a);
            pa_ra = pa * ia;
        }
        for (int k = 0; k < 9; k++) {
            const int nx = cx + kDX[k], ny = cy + kDY[k];
            if (nx < 0 || ny < 0 || nx >= g.ncx || ny >= g.ncy) continue;
            const int c = ny + nx * g.ncy;
            const float offx = (float)(-kDX[k]) * g.khf;
            const float offy = (float)(-kDY[k]) * g.khf;
            const int j0 = (int)__ldg(fstart + c), j1 = (int)__ldg(fstart + c + 1);
            for (int j = j0; j < j1; j++) {
                if (digest) {
                    const double2 rb = __ldg(NF.r + j);
                    const double drx = __dsub_rn(ra.x, rb.x), dry = __dsub_rn(ra.y, rb.y);
                    const double drs = __dsqrt_rn(__dadd_rn(__dmul_rn(drx, drx), __dmul_rn(dry, dry)));
                    if (__ddiv_rn(drs, P.hd) <= 2.0) {
                        const int nid = (int)fid[j];
                        dcount++;
                        dsum += nid;
                        dxor ^= nid;
                    }
                } else if constexpr (std::is_same<T, float>::value) {
                    const float2 lb = __ldg(NF.loc + j);
                    const float2 vb = __ldg(NF.v + j);
                    const float sb = __ldg(NF.rho + j);
                    const float pb = NF.p ? __ldg(NF.p + j) : eos(sb, P);
                    pair32((la.x - lb.x) + offx, (la.y - lb.y) + offy, -vb.x, -vb.y, rho_a, sa,
                           pa_ra, ia, P.rho0 + sb, sb, pb, P, acc);
                } else {
                    const double2 rb = __ldg(NF.r + j);
                    const double2 vb = __ldg(NF.v + j);
                    const double nrho = __ldg(NF.rho + j);
                    const double pb = NF.p ? __ldg(NF.p + j) : eos(nrho, P);
                    pair64(ra.x - rb.x, ra.y - rb.y, 0.0 - vb.x, 0.0 - vb.y, rho_a, nrho, pa, pb, P,
                           acc);
                }
            }
        }
        if (digest) {
            dig_count[w] = dcount;
            dig_sum[w] = dsum;
            dig_xor[w] = dxor;
            return;
        }
        if constexpr (std::is_same<T, float>::value) drho = (acc.cont - acc.diff) * P.m;
        else drho = acc.cont + acc.diff;
        Wl.drho[w] = drho;
    }
    if (correct) {
        const T sn = corrector_rho(Wl.rho_o[w], sa, drho, dt, P.rho0);
        Wl.rho[w] = sn;
        if constexpr (std::is_same<T, float>::value)
            if (RW.v) wall_record(RW, w, sn, P);
    }
}

// ------------------------------------------------------------- mDBC
__device__ __forceinline__ double det3(double a11, double a12, double a13, double a21,
                                       double a22, double a23, double a31, double a32,
                                       double a33) {
    return (a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 - a31 * a22 * a13 -
            a32 * a23 * a11 - a33 * a21 * a12);
}

// mDBC_compute_density_mdbcGeo (src/SPH_mDBC.h:9-50) with
// Kernel_density_approximation_MATRIX_mDBC (src/SPH_kernel_approx.h:1141-1343):
// one warp per wall particle; lanes split the fluid candidates of the ghost
// node's 3x3 cells, the 12 moment sums are reduced by shuffles, lane 0 solves
// the 3x3 system in FP64 (determinant threshold 0.001, Shepard and constant
// fall-backs) and clamps the density at 1000 (:43-44).
template <typename T>
__global__ void __launch_bounds__(kBlock)
k_mdbc(WallState<T> Wl, int nw, const uint32_t *__restrict__ fstart, Nbr<T> NF, Grid g,
       Phys<T> P) {
    pdl_enter();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nw) return;
    const uint32_t gk = Wl.gkey[warp];
    T s[12];
#pragma unroll
    for (int q = 0; q < 12; q++) s[q] = T(0);
    // s: 0 rhoWsum, 1 drhodx, 2 drhody, 3..11 a11 a12 a13 a21 a22 a23 a31 a32 a33
    if (gk < (uint32_t)g.ncells) {
        const int cx = (int)(gk / (uint32_t)g.ncy);
        const int cy = (int)gk - cx * g.ncy;
        const double2 gr = Wl.gnr[warp];
        float2 gl;
        if constexpr (std::is_same<T, float>::value) gl = Wl.gloc[warp];
        // gather candidate ranges of the 9 cells; lanes stride over the
        // concatenation in the reference's cell order
        int lo[9], len[9];
        int tot = 0;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int nx = cx + kDX[k], ny = cy + kDY[k];
            if (nx < 0 || ny < 0 || nx >= g.ncx || ny >= g.ncy) {
                lo[k] = 0;
                len[k] = 0;
                continue;
            }
            const int c = ny + nx * g.ncy;
            lo[k] = (int)__ldg(fstart + c);
            len[k] = (int)__ldg(fstart + c + 1) - lo[k];
            tot += len[k];
        }
        // FP32: lanes stride over the candidates; FP64: lane 0 alone, in the
        // reference's order, so the sums round exactly like the reference's
        const int t0 = std::is_same<T, float>::value ? lane : (lane == 0 ? 0 : tot);
        const int tstep = std::is_same<T, float>::value ? 32 : 1;
        for (int t = t0; t < tot; t += tstep) {
            int k = 0, rem = t;
            while (rem >= len[k]) {
                rem -= len[k];
                k++;
            }
            const int j = lo[k] + rem;
            if (NF.type && __ldg(NF.type + j) != 0) continue;  // fluid only (buffer zones)
            const T sb = __ldg(NF.rho + j);
            const T nrho = rho_full(sb, P.rho0);
            if constexpr (std::is_same<T, float>::value) {
                const float2 lb = __ldg(NF.loc + j);
                const float drx = (gl.x - lb.x) + (float)(-kDX[k]) * g.khf;
                const float dry = (gl.y - lb.y) + (float)(-kDY[k]) * g.khf;
                const float r2 = fmaf(drx, drx, dry * dry);
                if (!(r2 <= P.four_h2)) continue;
                float W, F;
                if (r2 == 0.f) {
                    W = P.awen;
                    F = 0.f;
                } else {
                    wendland32(r2, P, W, F, true);
                }
                const float V = P.m / nrho;
                s[0] += W;  // times m below
                s[1] = fmaf(drx, F, s[1]);
                s[2] = fmaf(dry, F, s[2]);
                const float WV = W * V, FV = F * V;
                s[3] += WV;
                s[4] = fmaf(drx, WV, s[4]);
                s[5] = fmaf(dry, WV, s[5]);
                s[6] = fmaf(drx, FV, s[6]);
                s[7] = fmaf(drx * drx, FV, s[7]);
                s[8] = fmaf(drx * dry, FV, s[8]);
                s[9] = fmaf(dry, FV, s[9]);
                s[10] = fmaf(dry * drx, FV, s[10]);
                s[11] = fmaf(dry * dry, FV, s[11]);
            } else {
                const double2 rb = __ldg(NF.r + j);
                const double drx = gr.x - rb.x, dry = gr.y - rb.y;
                const double drs = sqrt(drx * drx + dry * dry);
                double W, F;
                wendland64(drs, P.h, P.awen, P.bwen, W, F);
                const double m = P.m;
                s[0] += m * W;
                s[1] += drx * F * m;
                s[2] += dry * F * m;
                s[3] += W * (m / nrho);
                s[4] += drx * W * (m / nrho);
                s[5] += dry * W * (m / nrho);
                s[6] += drx * F * (m / nrho);
                s[7] += drx * drx * F * (m / nrho);
                s[8] += drx * dry * F * (m / nrho);
                s[9] += dry * F * (m / nrho);
                s[10] += dry * drx * F * (m / nrho);
                s[11] += dry * dry * F * (m / nrho);
            }
        }
        if constexpr (std::is_same<T, float>::value) {
#pragma unroll
            for (int q = 0; q < 12; q++) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], o);
            }
        }
    }
    if (lane != 0) return;
    double rhoWsum, drhodx, drhody;
    if constexpr (std::is_same<T, float>::value) {
        rhoWsum = (double)s[0] * (double)P.m;
        drhodx = (double)s[1] * (double)P.m;
        drhody = (double)s[2] * (double)P.m;
    } else {
        rhoWsum = s[0];
        drhodx = s[1];
        drhody = s[2];
    }
    const double a11 = s[3], a12 = s[4], a13 = s[5], a21 = s[6], a22 = s[7], a23 = s[8],
                 a31 = s[9], a32 = s[10], a33 = s[11];
    const double det = det3(a11, a12, a13, a21, a22, a23, a31, a32, a33);
    double dens;
    if (det > 0.001) {
        const double i11 = (a22 * a33 - a23 * a32) / det;
        const double i12 = -(a12 * a33 - a13 * a32) / det;
        const double i13 = (a12 * a23 - a13 * a22) / det;
        const double i21 = -(a21 * a33 - a23 * a31) / det;
        const double i22 = (a11 * a33 - a13 * a31) / det;
        const double i23 = -(a11 * a23 - a13 * a21) / det;
        const double i31 = (a21 * a32 - a22 * a31) / det;
        const double i32 = -(a11 * a32 - a12 * a31) / det;
        const double i33 = (a11 * a22 - a12 * a21) / det;
        const double dens_temp = rhoWsum * i11 + drhodx * i12 + drhody * i13;
        const double grx = -(rhoWsum * i21 + drhodx * i22 + drhody * i23);
        const double gry = -(rhoWsum * i31 + drhodx * i32 + drhody * i33);
        const auto gnd = Wl.gnd[warp];
        dens = (dens_temp + grx * (double)gnd.x + gry * (double)gnd.y);
    } else if (a11 > 0) {
        dens = rhoWsum / a11;
    } else {
        dens = 1000.;
    }
    if (dens < 1000.) dens = 1000.;
    Wl.rho[warp] = rho_stored_from_full<T>(dens, (double)P.rho0);
}

// ----------------------------------------------------- fused predictor
// Integrate_SymplecticPredictor (src/SPH_integration.h:266-287) out of place:
// reads the sorted state F, writes the predicted state to B (same order) and
// bins it.  The old state is F itself; the scatter copies it next to the
// predicted state.  Walls: rho_o = rho; rho += drho dt/2.
template <typename T>
__global__ void k_predict_bin(FluidState<T> F, const uint32_t *__restrict__ fstart, WallState<T> Wl,
                              int nw, Grid g, T dt, double2 *__restrict__ Br,
                              typename V2<T>::t *__restrict__ Bv, T *__restrict__ Brho,
                              uint32_t *__restrict__ key, uint32_t *__restrict__ slot,
                              uint32_t *__restrict__ counts, uint32_t *__restrict__ health) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        const T r = Wl.rho[i];
        Wl.rho_o[i] = r;
        Wl.rho[i] = r + Wl.drho[i] * dt * T(0.5);
        return;
    }
    const int f = i - nw;
    if (f >= n_live(fstart, g.ncells)) return;
    const double2 r = F.r[f];
    const auto v = F.v[f];
    const auto a = F.a[f];
    Brho[f] = F.rho[f] + F.drho[f] * dt * T(0.5);
    double2 rn;
    if constexpr (std::is_same<T, float>::value) {
        // FP32 displacement (v is FP32 already), one FP64 add per axis
        const float hdt = dt * 0.5f;
        rn = make_double2(r.x + (double)(v.x * hdt), r.y + (double)(v.y * hdt));
    } else {
        rn = make_double2(r.x + (double)v.x * (double)dt * 0.5, r.y + (double)v.y * (double)dt * 0.5);
    }
    Br[f] = rn;
    typename V2<T>::t nv;
    nv.x = v.x + a.x * dt * T(0.5);
    nv.y = v.y + a.y * dt * T(0.5);
    Bv[f] = nv;
    if (!(nv.x == nv.x) || !(nv.y == nv.y) || !is_finite_d(rn.x) || !is_finite_d(rn.y))
        atomicOr(health, kHealthNan);
    int cx, cy;
    const uint32_t k = cell_key(g, rn, F.key[f], &cx, &cy);
    if (k == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
    key[f] = k;
    slot[f] = atomicAdd(counts + k, 1u);
}

// Predictor of the fused FP32 step without re-binning: the predicted state
// goes to D in the current sorted order (cells, loc origins and fstart stay
// those of the last binning), the old state to O.  The cells stay exact for
// the pair set as long as every particle has moved less than `skin` per axis
// since its binning (a pair within 2h then still lies inside the 3 x 3 cell
// block, kh >= 2h + 2 skin); a larger move sets *rebuild (and, inside a CUDA
// graph, the conditional node `cond`), which runs the re-binning before the
// pair pass.
// the predictor of one fluid row f (shared with the mDBC-fused launch)
// Cells kept over several steps (the pair-record step): a re-binning is due
// once some particle has moved more than sqrt(sig2) from where it was binned
// (lbin: its cell-relative position then), or when the neighbour lists are
// stale (gen[0], the sorts so far, differs from gen[1], the sort they were
// built after).  With lbin == nullptr the test is the half step's own move
// against the skin.
struct KeepCells {
    const float2 *lbin;
    float sig2;
    const uint32_t *gen;
    uint32_t *clear;  // zeroed by the predictor (the corrector's need-sort flag), or nullptr
};

template <typename T>
__device__ __forceinline__ void predict_keep_fluid(int f, const FluidState<T> &F,
                                                   const uint32_t *__restrict__ fstart,
                                                   const Grid &g, T dt, const FluidState<T> &D,
                                                   const OldState<T> &O, float skin,
                                                   uint32_t *__restrict__ rebuild,
                                                   uint32_t *__restrict__ health,
                                                   cudaGraphConditionalHandle cond, int use_cond,
                                                   const KeepCells &kc,
                                                   const PairRec &R = PairRec{},
                                                   const Phys<T> *P = nullptr) {
    if (f == 0 && kc.clear) *kc.clear = 0u;
    if (f >= n_live(fstart, g.ncells)) return;
    const auto v = F.v[f];
    const auto a = F.a[f];
    const T s = F.rho[f];
    if (!R.e) {  // the corrector over pair records reads the old state from F itself
        O.r[f] = F.r[f];
        O.v[f] = v;
        O.rho[f] = s;
    }
    const float hdt = (float)dt * 0.5f;
    const float dx = (float)v.x * hdt, dy = (float)v.y * hdt;
    // the predicted FP64 position (r + dx) is formed only by a re-binning
    // (k_predict_r): the pair passes use the cell-relative position
    typename V2<T>::t nv;
    nv.x = v.x + a.x * dt * T(0.5);
    nv.y = v.y + a.y * dt * T(0.5);
    D.v[f] = nv;
    const T sp = s + F.drho[f] * dt * T(0.5);
    D.rho[f] = sp;
    const float2 l = F.loc[f];
    const float2 ln = make_float2(l.x + dx, l.y + dy);
    D.loc[f] = ln;
    const uint32_t key = F.key[f];
    D.key[f] = key;
    D.id[f] = F.id[f];
    if constexpr (std::is_same<T, float>::value) {
        if (R.e) {  // the pair records of the predicted state (kept cells)
            const float row = (float)(key % (uint32_t)g.ncy);
            const float ib = rcp_approx(P->rho0 + sp);
            R.e[f] = make_float4(ln.x, ln.y, row, ib);
            R.v[f] = make_float4(nv.x, nv.y, sp, eos(sp, *P) * ib);
        }
    }
    bool rebin;
    if (kc.lbin) {
        const float2 lb = kc.lbin[f];
        const float ex = ln.x - lb.x, ey = ln.y - lb.y;
        rebin = !(fmaf(ex, ex, ey * ey) <= kc.sig2) || __ldg(kc.gen) != __ldg(kc.gen + 1);
    } else {
        rebin = !(fabsf(dx) <= skin && fabsf(dy) <= skin);
    }
    if (rebin) {
        atomicOr(rebuild, 1u);
        if (use_cond) cudaGraphSetConditional(cond, 1u);
    }
    if (!(nv.x == nv.x) || !(nv.y == nv.y) || !(dx == dx) || !(dy == dy))
        atomicOr(health, kHealthNan);
}

// The fluid predictor of the fused FP32 step over U particles per thread
// (f0, f0 + stride, ...): every particle's loads are issued before the first
// store, so a thread keeps U particles' reads in flight (with one particle
// per thread the launch waits on memory latency with few bytes in flight).
// The arithmetic is predict_keep_fluid<float>'s, particle by particle.
template <int U>
__device__ __forceinline__ void predict_keep_fluid_f32(
    int f0, int stride, const FluidState<float> &F, const uint32_t *__restrict__ fstart,
    const Grid &g, float dt, const FluidState<float> &D, const OldState<float> &O, float skin,
    uint32_t *__restrict__ rebuild, uint32_t *__restrict__ health,
    cudaGraphConditionalHandle cond, int use_cond, const KeepCells &kc, const PairRec &R,
    const Phys<float> &P) {
    if (f0 == 0 && kc.clear) *kc.clear = 0u;
    const int nl = n_live(fstart, g.ncells);
    float2 v[U], a[U], l[U], lb[U];
    float s[U], ds[U];
    uint32_t key[U], id[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int f = f0 + u * stride;
        if (f < nl) {
            v[u] = F.v[f];
            a[u] = F.a[f];
            s[u] = F.rho[f];
            ds[u] = F.drho[f];
            l[u] = F.loc[f];
            key[u] = F.key[f];
            id[u] = F.id[f];
            lb[u] = kc.lbin ? kc.lbin[f] : make_float2(0.f, 0.f);
        }
    }
    const bool stale = kc.lbin && __ldg(kc.gen) != __ldg(kc.gen + 1);
    bool rebin = false, nan = false;
    const float hdt = dt * 0.5f;
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int f = f0 + u * stride;
        if (f >= nl) continue;
        if (!R.e) {  // the corrector over pair records reads the old state from F itself
            O.r[f] = F.r[f];
            O.v[f] = v[u];
            O.rho[f] = s[u];
        }
        const float dx = v[u].x * hdt, dy = v[u].y * hdt;
        const float2 nv = make_float2(v[u].x + a[u].x * dt * 0.5f, v[u].y + a[u].y * dt * 0.5f);
        D.v[f] = nv;
        const float sp = s[u] + ds[u] * dt * 0.5f;
        D.rho[f] = sp;
        const float2 ln = make_float2(l[u].x + dx, l[u].y + dy);
        D.loc[f] = ln;
        D.key[f] = key[u];
        D.id[f] = id[u];
        if (R.e) {  // the pair records of the predicted state (kept cells)
            const float row = (float)(key[u] % (uint32_t)g.ncy);
            const float ib = rcp_approx(P.rho0 + sp);
            R.e[f] = make_float4(ln.x, ln.y, row, ib);
            R.v[f] = make_float4(nv.x, nv.y, sp, eos(sp, P) * ib);
        }
        if (kc.lbin) {
            const float ex = ln.x - lb[u].x, ey = ln.y - lb[u].y;
            rebin |= !(fmaf(ex, ex, ey * ey) <= kc.sig2) || stale;
        } else {
            rebin |= !(fabsf(dx) <= skin && fabsf(dy) <= skin);
        }
        nan |= !(nv.x == nv.x) || !(nv.y == nv.y) || !(dx == dx) || !(dy == dy);
    }
    if (rebin) {
        atomicOr(rebuild, 1u);
        if (use_cond) cudaGraphSetConditional(cond, 1u);
    }
    if (nan) atomicOr(health, kHealthNan);
}

// the copy-back of a re-binning: every field of the sorted state S (and the
// old state carried in B) into the current buffers D and O, one launch over
// the rows in use (live and removed, fstart[ncells + 1]) instead of one copy
// per array over the whole capacity
template <typename T>
__global__ void k_copy_state(FluidState<T> D, FluidState<T> S, OldState<T> O, OldState<T> B,
                             const uint32_t *__restrict__ fstart, int ncells,
                             const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)__ldg(fstart + ncells + 1)) return;
    D.r[i] = S.r[i];
    D.v[i] = S.v[i];
    D.a[i] = S.a[i];
    D.rho[i] = S.rho[i];
    D.drho[i] = S.drho[i];
    D.p[i] = S.p[i];
    D.id[i] = S.id[i];
    D.key[i] = S.key[i];
    D.loc[i] = S.loc[i];
    if (D.type) D.type[i] = S.type[i];
    O.r[i] = B.r[i];
    O.v[i] = B.v[i];
    O.rho[i] = B.rho[i];
}

template <typename T>
__global__ void k_predict_keep(FluidState<T> F, const uint32_t *__restrict__ fstart,
                               WallState<T> Wl, int nw, Grid g, T dt, FluidState<T> D,
                               OldState<T> O, float skin, uint32_t *__restrict__ rebuild,
                               uint32_t *__restrict__ health, cudaGraphConditionalHandle cond,
                               int use_cond, KeepCells kc, PairRec RS, PairRec RW, Phys<T> P) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        const T r = Wl.rho[i];
        Wl.rho_o[i] = r;
        const T rp = r + Wl.drho[i] * dt * T(0.5);
        Wl.rho[i] = rp;
        if constexpr (std::is_same<T, float>::value)
            if (RW.v) wall_record(RW, i, rp, P);
        return;
    }
    predict_keep_fluid<T>(i - nw, F, fstart, g, dt, D, O, skin, rebuild, health, cond, use_cond,
                          kc, RS, &P);
}

// the predicted FP64 positions of a re-binning: r_old + (v_old dt/2), with
// the displacement formed in FP32 exactly as the predictor forms it, from
// the old state O; with `copy` the old state is also copied into C
template <typename T>
__global__ void k_predict_r(FluidState<T> D, OldState<T> O, OldState<T> C,
                            const uint32_t *__restrict__ fstart, int ncells, T dt,
                            const uint32_t *__restrict__ gate, int copy) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_live(fstart, ncells)) return;
    const double2 r = O.r[f];
    const auto v = O.v[f];
    const float hdt = (float)dt * 0.5f;
    const float dx = (float)v.x * hdt, dy = (float)v.y * hdt;
    D.r[f] = make_double2(r.x + (double)dx, r.y + (double)dy);
    if (copy) {
        C.r[f] = r;
        C.v[f] = v;
        C.rho[f] = O.rho[f];
    }
}

// gated re-binning of the predicted state: keys + histogram slots
template <typename T>
__global__ void k_bin_gated(const FluidState<T> X, const uint32_t *__restrict__ fstart, Grid g,
                            uint32_t *__restrict__ key, uint32_t *__restrict__ slot,
                            uint32_t *__restrict__ counts, uint32_t *__restrict__ health,
                            const uint32_t *__restrict__ gate, uint32_t *__restrict__ runs) {
    pdl_enter();
    if (gated_off(gate)) return;
    // `runs` counts the executions of a re-binning that a graph carries
    if (runs && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(runs, 1u);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live(fstart, g.ncells)) return;
    int cx, cy;
    const uint32_t k = cell_key(g, X.r[i], X.key[i], &cx, &cy);
    if (k == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
    key[i] = k;
    slot[i] = atomicAdd(counts + k, 1u);
}

// gated copy of a re-binned state back into the buffers the graph reads
template <typename T>
__global__ void k_copy_back(const FluidState<T> S, const double2 *__restrict__ or2,
                            const typename V2<T>::t *__restrict__ ov2, const T *__restrict__ orho2,
                            const uint32_t *__restrict__ fstart, int ncells, FluidState<T> D,
                            OldState<T> O, const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (int)fstart[ncells + 1]) return;
    D.r[j] = S.r[j];
    D.v[j] = S.v[j];
    D.rho[j] = S.rho[j];
    D.id[j] = S.id[j];
    D.key[j] = S.key[j];
    D.loc[j] = S.loc[j];
    O.r[j] = or2[j];
    O.v[j] = ov2[j];
    O.rho[j] = orho2[j];
}

// ------------------------------------------------------------ gathers
// dst[f] = src[perm[f]] for the sorted state (+ the old state when O != null);
// recomputes loc from the FP64 position and the key.
// --------------------------------------------------- host <-> device
// Per-index staging (SoA, double, indexed by original particle index) used by
// tsph_download / tsph_upload to present the state in the reference's order.
struct Staging {
    double2 *r, *v, *a;
    double *rho, *drho, *p;
    uint8_t *alive;
    int32_t *type = nullptr;  // systems with buffer zones: the particle type by index
};

template <typename T>
__global__ void k_export(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                         WallState<T> Wl, int nw, T rho0, Staging S, int mask) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        const uint32_t id = Wl.id[i];
        if (mask & 1) S.r[id] = Wl.r[i];
        if (mask & 2) S.v[id] = make_double2(0., 0.);
        if (mask & 4) S.a[id] = make_double2(0., 0.);
        if (mask & 8) S.rho[id] = rho_full64(Wl.rho[i], rho0);
        if (mask & 16) S.drho[id] = (double)Wl.drho[i];
        if (mask & 32) S.p[id] = (double)Wl.p[i];
        if (S.type) S.type[id] = 1;
        S.alive[id] = 1;
        return;
    }
    const int f = i - nw;
    if (f >= n_live(fstart, ncells)) return;
    const uint32_t id = F.id[f];
    if (F.key[f] == (uint32_t)ncells) {
        S.alive[id] = 0;
        return;
    }
    if (mask & 1) S.r[id] = F.r[f];
    if (mask & 2) {
        const auto v = F.v[f];
        S.v[id] = make_double2((double)v.x, (double)v.y);
    }
    if (mask & 4) {
        const auto a = F.a[f];
        S.a[id] = make_double2((double)a.x, (double)a.y);
    }
    if (mask & 8) S.rho[id] = rho_full64(F.rho[f], rho0);
    if (mask & 16) S.drho[id] = (double)F.drho[f];
    if (mask & 32) S.p[id] = (double)F.p[f];
    if (S.type) S.type[id] = F.type ? (int32_t)F.type[f] : 0;
    S.alive[id] = 1;
}

// number of live particles in the alive map: four flags per 32-bit word
// (the map is a cudaMalloc allocation, 256-byte aligned), a grid-stride
// loop, one atomic per block (one per warp on a single counter serialises
// in L2)
static __global__ void __launch_bounds__(kBlock) k_count_alive(const uint8_t *__restrict__ alive, int n,
                                                              uint32_t *__restrict__ count) {
    pdl_enter();
    __shared__ uint32_t part[kBlock / 32];
    const uint32_t *__restrict__ a4 = reinterpret_cast<const uint32_t *>(alive);
    const int nw = n >> 2;
    uint32_t c = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x)
        c += (uint32_t)__popc(__vcmpne4(__ldg(a4 + i), 0u)) >> 3;
    if (blockIdx.x == 0 && threadIdx.x < (n & 3)) c += alive[4 * nw + threadIdx.x] != 0 ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kBlock / 32; w++) t += part[w];
        if (t) atomicAdd(count, t);
    }
}

// `ntot` >= 0: a staged upload whose rows are the indices 0..ntot-1; applied
// only when every index is live, else TSPH_HEALTH_UPLOAD
template <typename T>
__global__ void k_import(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                         WallState<T> Wl, int nw, T rho0, Staging S, int mask, int ntot,
                         uint32_t *__restrict__ health) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (ntot >= 0 && n_live(fstart, ncells) + nw != ntot) {
        if (i == 0) atomicOr(health, kHealthUpload);
        return;
    }
    if (i < nw) {
        const uint32_t id = Wl.id[i];
        if (mask & 8) Wl.rho[i] = rho_stored_from_full<T>(S.rho[id], (double)rho0);
        if (mask & 16) Wl.drho[i] = (T)S.drho[id];
        if (mask & 32) Wl.p[i] = (T)S.p[id];
        return;
    }
    const int f = i - nw;
    if (f >= n_live(fstart, ncells)) return;
    if (F.key[f] == (uint32_t)ncells) return;
    const uint32_t id = F.id[f];
    if (mask & 1) F.r[f] = S.r[id];
    typename V2<T>::t t2;
    if (mask & 2) {
        const double2 v = S.v[id];
        t2.x = (T)v.x;
        t2.y = (T)v.y;
        F.v[f] = t2;
    }
    if (mask & 4) {
        const double2 a = S.a[id];
        t2.x = (T)a.x;
        t2.y = (T)a.y;
        F.a[f] = t2;
    }
    if (mask & 8) F.rho[f] = rho_stored_from_full<T>(S.rho[id], (double)rho0);
    if (mask & 16) F.drho[f] = (T)S.drho[id];
    if (mask & 32) F.p[f] = (T)S.p[id];
}

// FP64 totals over live fluid: mass, kinetic energy, momentum (block partials)
template <typename T>
__global__ void k_totals(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells, double m,
                         double *__restrict__ out) {
    pdl_enter();
    __shared__ double sh[4][kBlock / 32];
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    if (f < n_live(fstart, ncells) && F.key[f] != (uint32_t)ncells) {
        const auto v = F.v[f];
        const double vx = v.x, vy = v.y;
        v0 = m;
        v1 = 0.5 * m * (vx * vx + vy * vy);
        v2 = m * vx;
        v3 = m * vy;
    }
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_down_sync(0xffffffffu, v0, o);
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
        v2 += __shfl_down_sync(0xffffffffu, v2, o);
        v3 += __shfl_down_sync(0xffffffffu, v3, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = v0;
        sh[1][wid] = v1;
        sh[2][wid] = v2;
        sh[3][wid] = v3;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0;
        for (int w = 0; w < kBlock / 32; w++) s += sh[threadIdx.x][w];
        out[(size_t)blockIdx.x * 4 + threadIdx.x] = s;
    }
}

// RemoveParticlesOutOfDomain's erase over the corrector's candidates (one
// block; before the sort): all parities are read before any erase is
// written.  A candidate that survives keeps the cell it was binned into; one
// outside the cell grid cannot be binned and is dropped as escaped.
constexpr int kResolveThreads = 1024;
static __global__ void __launch_bounds__(kResolveThreads)
k_resolve_removal(Removal rm, uint8_t *__restrict__ dead, uint32_t *__restrict__ key,
                  uint32_t *__restrict__ slot, uint32_t *__restrict__ counts, int ncells,
                  uint32_t *__restrict__ health, const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    __shared__ uint8_t erase[kRemovalCap];
    const int n = (int)min(*rm.count, (uint32_t)rm.cap);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int id = (int)rm.ids[rm.list[k]];
        int c = 0;
        for (int j = id - 1; j >= 0; j--) {
            if (dead[j]) continue;
            if (!rm.cand[j]) break;
            c++;
        }
        erase[k] = (c & 1) == 0 ? 1 : 0;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const uint32_t row = rm.list[k];
        uint32_t kk = key[row];
        if (erase[k]) {
            kk = (uint32_t)ncells;
            dead[rm.ids[row]] = 1;
            atomicOr(health, kHealthRemoved);
        } else if (kk == (uint32_t)ncells) {
            dead[rm.ids[row]] = 1;
            atomicOr(health, kHealthEscaped);
        }
        key[row] = kk;
        slot[row] = atomicAdd(counts + kk, 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) rm.cand[rm.ids[rm.list[k]]] = 0;
    if (threadIdx.x == 0) *rm.count = 0u;
}

}  // namespace tsph
