// tsph_graph.cuh -- the particle graph for the learned surrogate: every
// particle (walls first, then the live fluid in its sorted order) is a node,
// every pair within the kernel support (0 < r <= 2h, the pair set of the
// SPH step) is an edge, stored as a fixed-width neighbour table (ELL: K
// slots per node, unused slots -1).  And the surrogate's update of the fluid
// state after a window of k SPH steps.
#pragma once

#include "tsph_kernels.cuh"

namespace tsph {

// one thread per node; candidates from the 3 x 3 cell block (walls and
// fluid), FP32 cell-local distances as in the pair kernels
template <typename T>
__global__ void k_graph_export(FluidState<T> F, const uint32_t *__restrict__ fstart,
                               const uint32_t *__restrict__ wstart, WallState<T> Wl, int nw,
                               Grid g, T rho0, float four_h2, int K, double2 *__restrict__ pos,
                               float2 *__restrict__ vel, float *__restrict__ srho,
                               float *__restrict__ wall, int32_t *__restrict__ id,
                               int32_t *__restrict__ deg, int32_t *__restrict__ nbr,
                               float2 *__restrict__ acc, float *__restrict__ rate,
                               uint32_t *__restrict__ overflow) {
    pdl_enter();
    const int node = blockIdx.x * blockDim.x + threadIdx.x;
    const int nl = n_live(fstart, g.ncells);
    if (node >= nw + nl) return;
    const bool is_wall = node < nw;
    const int f = node - nw;
    const uint32_t key = is_wall ? Wl.key[node] : F.key[f];
    const int cx = (int)(key / (uint32_t)g.ncy), cy = (int)key - cx * g.ncy;
    const float2 la = is_wall ? Wl.loc[node] : F.loc[f];
    pos[node] = is_wall ? Wl.r[node] : F.r[f];
    if (is_wall) {
        vel[node] = make_float2(0.f, 0.f);
        srho[node] = (float)(rho_full64(Wl.rho[node], rho0) - (double)rho0);
    } else {
        vel[node] = make_float2((float)F.v[f].x, (float)F.v[f].y);
        srho[node] = (float)(rho_full64(F.rho[f], rho0) - (double)rho0);
    }
    wall[node] = is_wall ? 1.f : 0.f;
    id[node] = (int32_t)(is_wall ? Wl.id[node] : F.id[f]);
    if (acc) acc[node] = is_wall ? make_float2(0.f, 0.f)
                                 : make_float2((float)F.a[f].x, (float)F.a[f].y);
    if (rate) rate[node] = is_wall ? 0.f : (float)F.drho[f];
    int cnt = 0;
    int32_t *row = nbr + (size_t)node * K;
    for (int dxi = -1; dxi <= 1; dxi++) {
        const int col = cx + dxi;
        if (col < 0 || col >= g.ncx) continue;
        for (int dyi = -1; dyi <= 1; dyi++) {
            const int rr = cy + dyi;
            if (rr < 0 || rr >= g.ncy) continue;
            const int c = col * g.ncy + rr;
            const float ox = (float)dxi * g.khf, oy = (float)dyi * g.khf;
            for (int kind = 0; kind < 2; kind++) {
                const uint32_t *st = kind ? fstart : wstart;
                for (int j = (int)st[c]; j < (int)st[c + 1]; j++) {
                    const int other = kind ? nw + j : j;
                    if (other == node) continue;
                    const float2 lb = kind ? F.loc[j] : Wl.loc[j];
                    // the distance as the lower-numbered node sees it, so that
                    // both ends of a pair make the same test: the edge set is
                    // exactly symmetric (the backward pass relies on it)
                    float dx, dy;
                    if (node < other) {
                        dx = (la.x - ox) - lb.x;
                        dy = (la.y - oy) - lb.y;
                    } else {
                        dx = (lb.x + ox) - la.x;
                        dy = (lb.y + oy) - la.y;
                    }
                    const float r2 = fmaf(dx, dx, dy * dy);
                    if (!(r2 > 0.f && r2 <= four_h2)) continue;
                    if (cnt < K) row[cnt] = other;
                    cnt++;
                }
            }
        }
    }
    if (cnt > K) atomicOr(overflow, 1u);
    deg[node] = cnt < K ? cnt : K;
    for (int k = cnt; k < K; k++) row[k] = -1;
}

// sums over the fluid nodes of (y0, y1) and their count into out[0..2]
static __global__ void k_fluid_sum2(const uint32_t *__restrict__ fstart, int ncells, int nw,
                             const float *__restrict__ y, double *__restrict__ out) {
    pdl_enter();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0, b = 0, c = 0;
    if (f < n_live(fstart, ncells)) {
        const size_t node = (size_t)(nw + f);
        a = y[3 * node];
        b = y[3 * node + 1];
        c = 1;
    }
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
        c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    // one atomic per block (blockDim.x = kBlock)
    __shared__ double red[3][kBlock / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = a;
        red[1][w] = b;
        red[2][w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kBlock / 32; k++) {
            a += red[0][k];
            b += red[1][k];
            c += red[2][k];
        }
        if (c > 0) {
            atomicAdd(out, a);
            atomicAdd(out + 1, b);
            atomicAdd(out + 2, c);
        }
    }
}

// the start-of-window terms of the window check, by particle index
struct WindowRef {
    double *rho;    // rho at the window start
    double2 *v;     // v at the window start
    float *drho;    // d(rho)/dt of the forces pass at the window start
    float2 *a;      // a of that pass
};

// the surrogate's window update of the fluid (node nw + f is fluid row f of
// the export), phase 0 (explicit), 1 (kick) or 2 (drift):
//   0: v_new = v + add_rates kdt a + su (y0, y1),  rho += add_rates kdt drho + ss y2,
//      r += kdt (v + v_new) / 2
//   1: v_new as in 0; rho, r unchanged
//   2: rho += add_rates kdt drho + ss y2 (drho of the pass after the kick),
//      r += kdt (v_start + v) / 2
template <typename T>
__global__ void k_apply_update(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                               int nw, const float *__restrict__ y, float su, float ss, double kdt,
                               int add_rates, int phase, const double *__restrict__ ysum,
                               T rho0, WindowRef ref, uint32_t *__restrict__ health) {
    pdl_enter();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_live(fstart, ncells)) return;
    const int node = nw + f;
    const uint32_t pid = F.id[f];
    float y0 = y[3 * (size_t)node], y1 = y[3 * (size_t)node + 1];
    const float y2 = y[3 * (size_t)node + 2];
    if (ysum && ysum[2] > 0) {  // less the fluid mean (a correction without momentum)
        y0 -= (float)(ysum[0] / ysum[2]);
        y1 -= (float)(ysum[1] / ysum[2]);
    }
    const T kr = add_rates ? (T)kdt : T(0);
    const auto v0 = F.v[f];
    if (phase == 2) {
        F.rho[f] = F.rho[f] + (kr * F.drho[f] + (T)(ss * y2));
        const double2 vs = ref.v[pid];
        const double2 r = F.r[f];
        F.r[f] = make_double2(r.x + kdt * 0.5 * (vs.x + (double)v0.x),
                              r.y + kdt * 0.5 * (vs.y + (double)v0.y));
        if (!(F.rho[f] == F.rho[f])) atomicOr(health, kHealthNan);
        return;
    }
    const auto a0 = F.a[f];
    const T dr0 = F.drho[f];
    ref.rho[pid] = rho_full64(F.rho[f], rho0);
    ref.v[pid] = make_double2((double)v0.x, (double)v0.y);
    ref.drho[pid] = (float)dr0;
    ref.a[pid] = make_float2((float)a0.x, (float)a0.y);
    typename V2<T>::t v1;
    v1.x = v0.x + kr * a0.x + (T)(su * y0);
    v1.y = v0.y + kr * a0.y + (T)(su * y1);
    F.v[f] = v1;
    if (!(v1.x == v1.x) || !(v1.y == v1.y)) atomicOr(health, kHealthNan);
    if (phase == 1) return;
    F.rho[f] = F.rho[f] + (kr * dr0 + (T)(ss * y2));  // rho - rho0 (FP32) or rho (FP64)
    const double2 r = F.r[f];
    F.r[f] = make_double2(r.x + kdt * 0.5 * ((double)v0.x + (double)v1.x),
                          r.y + kdt * 0.5 * ((double)v0.y + (double)v1.y));
    if (!(F.rho[f] == F.rho[f])) atomicOr(health, kHealthNan);
}

// the check of a window after a forces pass at its end state: per fluid
// particle e = rho - (rho_0 + kdt (drho_0 + drho_1) / 2) and
// ev = v - (v_0 + kdt (a_0 + a_1) / 2); out[0] max |e| (as the bits of a
// non-negative double), out[1] sum e^2, out[2..3] sum ev, out[4] sum
// |kdt (a_0 + a_1) / 2| (diagnostic), out[5] count, out[6] (float bits of
// max |e|) << 32 | its particle index
template <typename T>
__global__ void k_window_check(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                               double kdt, T rho0, WindowRef ref, double *__restrict__ out) {
    pdl_enter();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0, ex = 0, ey = 0, dvc = 0, one = 0;
    unsigned long long arg = 0ull;
    if (f < n_live(fstart, ncells) && F.key[f] < (uint32_t)ncells) {
        const uint32_t pid = F.id[f];
        const double rc = ref.rho[pid] + 0.5 * kdt * ((double)ref.drho[pid] + (double)F.drho[f]);
        e = fabs(rho_full64(F.rho[f], rho0) - rc);
        const double2 v0 = ref.v[pid];
        const float2 a0 = ref.a[pid];
        const auto a1 = F.a[f];
        const double cx = 0.5 * kdt * ((double)a0.x + (double)a1.x);
        const double cy = 0.5 * kdt * ((double)a0.y + (double)a1.y);
        ex = (double)F.v[f].x - (v0.x + cx);
        ey = (double)F.v[f].y - (v0.y + cy);
        dvc = sqrt(cx * cx + cy * cy);
        one = 1;
        arg = ((unsigned long long)__float_as_uint((float)e) << 32) | pid;
    }
    double mx = e, sq = e * e;
    for (int o = 16; o; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sq += __shfl_xor_sync(0xffffffffu, sq, o);
        ex += __shfl_xor_sync(0xffffffffu, ex, o);
        ey += __shfl_xor_sync(0xffffffffu, ey, o);
        dvc += __shfl_xor_sync(0xffffffffu, dvc, o);
        one += __shfl_xor_sync(0xffffffffu, one, o);
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, arg, o);
        arg = w > arg ? w : arg;
    }
    // one set of atomics per block (blockDim.x = kBlock)
    __shared__ double red[6][kBlock / 32];
    __shared__ unsigned long long rarg[kBlock / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[0][w] = mx;
        red[1][w] = sq;
        red[2][w] = ex;
        red[3][w] = ey;
        red[4][w] = dvc;
        red[5][w] = one;
        rarg[w] = arg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kBlock / 32; k++) {
            mx = fmax(mx, red[0][k]);
            sq += red[1][k];
            ex += red[2][k];
            ey += red[3][k];
            dvc += red[4][k];
            one += red[5][k];
            arg = rarg[k] > arg ? rarg[k] : arg;
        }
        if (one > 0) {
            atomicMax(reinterpret_cast<unsigned long long *>(out), (unsigned long long)__double_as_longlong(mx));
            atomicAdd(out + 1, sq);
            atomicAdd(out + 2, ex);
            atomicAdd(out + 3, ey);
            atomicAdd(out + 4, dvc);
            atomicAdd(out + 5, one);
            atomicMax(reinterpret_cast<unsigned long long *>(out + 6), arg);
        }
    }
}

}  // namespace tsph
