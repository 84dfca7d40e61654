// tsph_probes.cuh -- the case drivers' probes on the device: the water level
// of src/SPH_water_level.h:84-150 (Water_Elevation, Water_Elevation_inverse)
// and the Shepard point fields of src/testing.h:6-149 behind
// Pressure_in_point (src/SPH_measure_pressure.h:6-15), plus the water front
// (the largest x of the fluid below a height; the reference computes none).
//
// The probes run in FP64 with the reference's Wendland roundings over the
// 3 x 3 cell block of the probe point, fluid and walls alike (the reference
// has no type filter there); only the order of the sums differs.
#pragma once

#include "tsph_kernels.cuh"

namespace tsph {

template <typename T> struct ProbeSrc {
    const double2 *fr;
    const typename V2<T>::t *fv;
    const T *frho, *fp;
    const double2 *wr;
    const T *wrho, *wp;
    const uint32_t *fstart, *wstart;
    Grid g;
    double h, awen, bwen, m, rho_off;  // rho_off: rho0 when the density is stored as rho - rho0
};

// cell of a probe point: the reference's (int)((x - x_0 + of)/kh) through the
// exact boundary tables; -1 outside the grid
static __device__ __forceinline__ bool probe_cell(const Grid &g, double x, double y, int &cx, int &cy) {
    cx = axis_cell(g.ax, x, g.ncx >> 1);
    cy = axis_cell(g.ay, y, g.ncy >> 1);
    return cx >= 0 && cy >= 0 && cx < g.ncx && cy < g.ncy;
}

// Sum_kernel_function (src/SPH_water_level.h:6-80): sum of m W / rho
template <typename T>
__device__ double kernel_volume(const ProbeSrc<T> &S, double x, double y) {
    int cx, cy;
    if (!probe_cell(S.g, x, y, cx, cy)) return 0.0;
    double mw = 0.0;
    for (int dxi = -1; dxi <= 1; dxi++) {
        const int col = cx + dxi;
        if (col < 0 || col >= S.g.ncx) continue;
        for (int dyi = -1; dyi <= 1; dyi++) {
            const int row = cy + dyi;
            if (row < 0 || row >= S.g.ncy) continue;
            const int c = col * S.g.ncy + row;
            for (int kind = 0; kind < 2; kind++) {
                const uint32_t *st = kind ? S.fstart : S.wstart;
                const double2 *rr = kind ? S.fr : S.wr;
                const T *rh = kind ? S.frho : S.wrho;
                for (int j = (int)st[c]; j < (int)st[c + 1]; j++) {
                    const double2 r = rr[j];
                    const double dx = x - r.x, dy = y - r.y;
                    double W, F;
                    wendland64(sqrt(dx * dx + dy * dy), S.h, S.awen, S.bwen, W, F);
                    mw += S.m * W / ((double)rh[j] + S.rho_off);
                }
            }
        }
    }
    return mw;
}

// grid (gauges, chunks): CTA (g, c) tests the samples [c kWlChunk,
// (c + 1) kWlChunk) of gauge g (the reference's growing-step sequence,
// accumulated on the host in FP64) in rounds of 256; the first index where
// the kernel volume crosses 0.5 (<= 0.5 upwards, >= 0.5 downwards) is folded
// into first[g] with atomicMin (the host fills first[] with 0x7f7f7f7f)
constexpr int kWlChunk = 1024;

template <typename T>
__global__ void __launch_bounds__(256)
k_water_level(ProbeSrc<T> S, const double *__restrict__ gx, const int *__restrict__ inverse,
              const double *__restrict__ ys, const int *__restrict__ yoff,
              int *__restrict__ first) {
    __shared__ int best;
    const int gauge = blockIdx.x;
    const int n = yoff[gauge + 1] - yoff[gauge];
    const int c0 = (int)blockIdx.y * kWlChunk;
    if (c0 >= n) return;  // whole CTA: nothing in this chunk
    const int c1 = min(n, c0 + kWlChunk);
    const double *y = ys + yoff[gauge];
    const double x = gx[gauge];
    const bool inv = inverse[gauge] != 0;
    if (threadIdx.x == 0) best = 0x7fffffff;
    __syncthreads();
    for (int base = c0; base < c1; base += blockDim.x) {
        const int i = base + (int)threadIdx.x;
        if (i < c1) {
            const double mw = kernel_volume(S, x, y[i]);
            if (inv ? (mw >= 0.5) : (mw <= 0.5)) atomicMin(&best, i);
        }
        __syncthreads();
        if (best != 0x7fffffff) break;  // block-uniform: read after the barrier
        __syncthreads();
    }
    if (threadIdx.x == 0 && best != 0x7fffffff) atomicMin(first + gauge, best);
}

// one warp per point: Kernel_velocity_approximation_TEST's sums, then
// {rho, p, vx, vy} = sum f W / sum W where the kernel volume exceeds 0.5
template <typename T>
__global__ void k_point_fields(ProbeSrc<T> S, const double *__restrict__ xy, int npts,
                               double *__restrict__ out) {
    pdl_enter();
    const int pt = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pt >= npts) return;
    const double x = xy[2 * pt], y = xy[2 * pt + 1];
    double s[6] = {0, 0, 0, 0, 0, 0};  // W, vx W, vy W, rho W, p W, m W / rho
    int cx, cy;
    if (probe_cell(S.g, x, y, cx, cy)) {
        for (int e = 0; e < 9; e++) {
            const int col = cx + e / 3 - 1, row = cy + e % 3 - 1;
            if (col < 0 || col >= S.g.ncx || row < 0 || row >= S.g.ncy) continue;
            const int c = col * S.g.ncy + row;
            for (int kind = 0; kind < 2; kind++) {
                const uint32_t *st = kind ? S.fstart : S.wstart;
                const int j0 = (int)st[c], j1 = (int)st[c + 1];
                for (int j = j0 + lane; j < j1; j += 32) {
                    const double2 r = kind ? S.fr[j] : S.wr[j];
                    const double dx = x - r.x, dy = y - r.y;
                    double W, F;
                    wendland64(sqrt(dx * dx + dy * dy), S.h, S.awen, S.bwen, W, F);
                    const double rho = (double)(kind ? S.frho[j] : S.wrho[j]) + S.rho_off;
                    const double p = (double)(kind ? S.fp[j] : S.wp[j]);
                    double vx = 0.0, vy = 0.0;
                    if (kind) {
                        vx = (double)S.fv[j].x;
                        vy = (double)S.fv[j].y;
                    }
                    s[0] += W;
                    s[1] += vx * W;
                    s[2] += vy * W;
                    s[3] += rho * W;
                    s[4] += p * W;
                    s[5] += S.m * W / rho;
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 6; q++)
        for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    if (lane == 0) {
        double rho = 0.0, p = 0.0, vx = 0.0, vy = 0.0;
        if (s[5] > 0.5) {
            vx = 0.0 + s[1] / s[0];
            vy = 0.0 + s[2] / s[0];
            rho = 0.0 + s[3] / s[0];
            p = 0.0 + s[4] / s[0];
        }
        if (s[0] == 0.0) vx = vy = 0.0;
        out[4 * pt] = rho;
        out[4 * pt + 1] = p;
        out[4 * pt + 2] = vx;
        out[4 * pt + 3] = vy;
    }
}

// largest x of the live fluid with y <= y_max (ordered bits, atomicMax)
static __global__ void k_water_front(const double2 *__restrict__ fr, const uint32_t *__restrict__ fstart,
                              int ncells, double y_max, unsigned long long *__restrict__ best) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long v = 0ull;
    if (i < (int)fstart[ncells]) {
        const double2 r = fr[i];
        if (r.y <= y_max && is_finite_d(r.x))
            v = (unsigned long long)(ordered_bits(r.x) ^ (long long)0x8000000000000000ULL);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    if ((threadIdx.x & 31) == 0 && v) atomicMax(best, v);
}

}  // namespace tsph
