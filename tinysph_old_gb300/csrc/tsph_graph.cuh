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
                               uint32_t *__restrict__ overflow) {
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

// the surrogate's window update of the fluid (node nw + f is fluid row f of
// the export): v += dv, rho - rho0 += ds, r += k dt (v_old + v_new) / 2
template <typename T>
__global__ void k_apply_update(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                               int nw, const float *__restrict__ du, const float *__restrict__ dv,
                               const float *__restrict__ ds, double kdt,
                               uint32_t *__restrict__ health) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_live(fstart, ncells)) return;
    const int node = nw + f;
    const auto v0 = F.v[f];
    typename V2<T>::t v1;
    v1.x = v0.x + (T)du[node];
    v1.y = v0.y + (T)dv[node];
    F.v[f] = v1;
    F.rho[f] = F.rho[f] + (T)ds[node];  // rho - rho0 in the FP32 build, rho in FP64: the same increment
    const double2 r = F.r[f];
    F.r[f] = make_double2(r.x + kdt * 0.5 * ((double)v0.x + (double)v1.x),
                          r.y + kdt * 0.5 * ((double)v0.y + (double)v1.y));
    if (!(v1.x == v1.x) || !(v1.y == v1.y)) atomicOr(health, kHealthNan);
}

}  // namespace tsph
