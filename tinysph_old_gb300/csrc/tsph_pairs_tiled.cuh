// tsph_pairs_tiled.cuh -- the FP32 pair loop as a shared-memory tiled gather
// kernel (the production path of Compute_Forces, src/SPH_interaction.h:8-149,
// fused with the symplectic corrector of src/SPH_integration.h:289-309).
//
// Work decomposition: a CTA takes 128 consecutive fluid particles of the
// cell-sorted state (their cells are consecutive rows of one or two grid
// columns).  For each window of at most kTileRows target rows of one column it
//   1. stages the 3 x (rows + 2) neighbour cells (fluid and walls) into shared
//      memory, all of a thread's loads issued before its stores: FP32
//      position, x relative to the window's centre column and y relative to
//      the particle's own cell (so r_a - r_b keeps ~1e-7 relative precision
//      without FP64), velocity, rho - rho0, p/rho and 1/rho (the EOS and the
//      reciprocal done once per staged particle instead of once per pair);
//   2. phase 1: every thread walks, per neighbour column, the staged ranges
//      of the rows below, at and above its own (contiguous and sorted by y,
//      so the rows above and below stop once |dy| passes the reach) and
//      appends the in-support neighbours (r <= 2h, the particle itself
//      excluded) to a private list of (staged index, row code) entries;
//   3. phase 2: every thread evaluates the WCSPH pair terms over its list, so
//      the expensive arithmetic runs with nearly all lanes active (a plain
//      candidate loop would execute it for ~80 candidates with ~30% of the
//      lanes useful).
// A window whose neighbour block exceeds the shared-memory capacity falls
// back to reading the neighbours from global memory (same arithmetic).
#pragma once

#include "tsph_kernels.cuh"

namespace tsph {

constexpr int kTileT = 128;     // targets per CTA
constexpr int kTileRows = 16;   // max target rows per window (halved while the block is too big)
// Two tile shapes, both 8 CTAs/SM (under 27.5 KB of shared memory each):
// 608 staged neighbours + 36 list entries per target (h ~ 1.4 dp: ~24
// neighbours), or 512 + 44 (h ~ 1.5 dp: ~28 neighbours); the engine times both
// on its own particles and keeps the faster (a target whose list would
// overflow takes the global-memory path).
template <int CAP, int LIST> struct TileShape {
    static constexpr int cap = CAP, list = LIST;
};
typedef TileShape<608, 36> TileWide;
typedef TileShape<512, 44> TileDeep;

// 8 CTAs of 128 threads per SM: 28 B per staged neighbour + 72 B of list per
// target keep a CTA under 27.5 KB of shared memory
template <class SH> struct TileSmem {
    float2 loc[SH::cap];
    float4 vs[SH::cap];   // {vx, vy, rho - rho0, p/rho}
    float inv[SH::cap];   // 1/rho
    int foff[3][kTileRows + 3];
    int woff[3][kTileRows + 3];
    float offy[4];  // y offset of a neighbour row: below, own, above (list code 0, 1, 2)
    uint16_t list[SH::list * kTileT];
};

// Pair terms with the constant factors (m, bwen/h, k_psi) applied once per
// target by the caller: a = -m bwen_h sum dr w^3 (P_a I_b + P_b I_a + Pi),
// drho = m bwen_h (sum w^3 dr.dv - k_psi sum psi r^2 w^3 I_b).
struct Acc4 {
    float ax, ay, cont, diff;
};

struct TileConst {
    float neg_half_inv_h;  // -0.5 / h
    float eps_h2, four_h2;
    float k_av;             // -2 alpha c0 h: Pi = k_av dr.dv / ((r^2 + eps h^2)(rho_a + rho_b))
    float c1, c2;           // rho0((1 + x)^(1/7) - 1) ~ dy (c1 + c2 dy), x = xg dy
    float two_rho0;
    float reach;            // |dy| beyond which the y-sorted rows above / below stop
};

__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Ra2 = 2 rho0 + (rho_a - rho0), so rho_a + rho_b = Ra2 + sb.  With CLAMP the
// kernel factor (1 - q/2) is clamped at 0, so a pair beyond 2h adds exactly
// zero to every sum (lists that hold neighbours up to a larger radius).
template <bool CLAMP = false>
__device__ __forceinline__ void pair_terms(float dx, float dy, float dvx, float dvy, float sa,
                                           float Pa, float Ia, float Ra2, float sb, float Pb,
                                           float Ib, const TileConst &K, Acc4 &acc) {
    const float dy2 = dy * dy;
    const float r2 = fmaf(dx, dx, dy2);
    float w1 = fmaf(sqrt_approx(r2), K.neg_half_inv_h, 1.f);
    if (CLAMP) w1 = fmaxf(w1, 0.f);
    const float w3 = w1 * w1 * w1;
    const float drdv = fmaf(dx, dvx, dy * dvy);
    const float inv_den = rcp_approx(r2 + K.eps_h2);
    float pterm = fmaf(Pa, Ib, Pb * Ia);
    if (drdv < 0.f) {
        // artificial viscosity with the mean density 0.5 (rho_a + rho_b)
        pterm = fmaf(K.k_av * drdv, inv_den * rcp_approx(Ra2 + sb), pterm);
    }
    const float coef = w3 * pterm;
    acc.ax = fmaf(-dx, coef, acc.ax);
    acc.ay = fmaf(-dy, coef, acc.ay);
    acc.cont = fmaf(w3, drdv, acc.cont);
    // (rho_b - rho_a) - rho0((1 + x)^(1/7) - 1) with x = 7 g dy / c0^2
    const float psi = fmaf(-K.c2, dy2, fmaf(-K.c1, dy, sb - sa)) * inv_den;
    acc.diff = fmaf(psi * r2, w3 * Ib, acc.diff);
}

// per-particle derived quantities of a neighbour: {vx, vy, s, p/rho} and 1/rho
__device__ __forceinline__ float4 staged_vs(float2 v, float s, float p, float inv) {
    return make_float4(v.x, v.y, s, p * inv);
}

// all in-support neighbours of one target straight from global memory (the
// path for windows whose neighbour block does not fit in shared memory, and
// for targets whose list overflows)
template <bool STORED_P>
__device__ __forceinline__ void target_global(const FluidState<float> &F, const uint32_t *fstart,
                                              const uint32_t *wstart, const WallState<float> &Wl,
                                              const Grid &g, const Phys<float> &P,
                                              const TileConst &K, int i, int cx, int cy, float2 la,
                                              float2 va, float sa, float Pa, float Ia, float Ra2,
                                              Acc4 &acc) {
    for (int dxi = 0; dxi < 3; dxi++) {
        const int col = cx + dxi - 1;
        if (col < 0 || col >= g.ncx) continue;
        for (int dyi = 0; dyi < 3; dyi++) {
            const int row = cy + dyi - 1;
            if (row < 0 || row >= g.ncy) continue;
            const int c = col * g.ncy + row;
            const float ox = (float)(1 - dxi) * g.khf, oy = (float)(1 - dyi) * g.khf;
            for (int kind = 0; kind < 2; kind++) {
                const int j0 = (int)__ldg((kind == 0 ? wstart : fstart) + c);
                const int j1 = (int)__ldg((kind == 0 ? wstart : fstart) + c + 1);
                for (int j = j0; j < j1; j++) {
                    if (kind == 1 && j == i) continue;
                    const float2 lb = __ldg((kind == 0 ? Wl.loc : F.loc) + j);
                    const float dx = (la.x + ox) - lb.x, dy = (la.y + oy) - lb.y;
                    const float r2 = fmaf(dx, dx, dy * dy);
                    if (!(r2 <= K.four_h2 && r2 > 0.f)) continue;
                    const float s = __ldg((kind == 0 ? Wl.rho : F.rho) + j);
                    const float p = STORED_P ? __ldg((kind == 0 ? Wl.p : F.p) + j) : eos(s, P);
                    const float ib = rcp_approx(P.rho0 + s);
                    const float2 vb = kind == 0 ? make_float2(0.f, 0.f) : __ldg(F.v + j);
                    pair_terms(dx, dy, va.x - vb.x, va.y - vb.y, sa, Pa, Ia, Ra2, s, p * ib, ib, K,
                               acc);
                }
            }
        }
    }
}

template <int MODE, bool STORED_P, class SH>
__global__ void __launch_bounds__(kTileT, 8)
k_pairs_tiled(FluidState<float> F, const uint32_t *__restrict__ fstart,
              const uint32_t *__restrict__ wstart, WallState<float> Wl, Grid g, Phys<float> P,
              TileConst K, OldState<float> O, float dt, PairOut out,
              uint32_t *__restrict__ health) {
    pdl_enter();
    __shared__ TileSmem<SH> sm;
    const int tid = threadIdx.x;
    const int ncy = g.ncy;
    const int nl = n_live(fstart, g.ncells);
    const int t0 = blockIdx.x * kTileT;
    if (t0 >= nl) return;
    const int t1 = min(t0 + kTileT, nl);
    if (tid < 4) sm.offy[tid] = tid < 3 ? (float)(1 - tid) * g.khf : 0.f;
    const float khf = g.khf;
    // rows above / below are sorted by y (as of the last binning): stop once
    // |dy| > K.reach = 2h (+ rounding margin, + twice the skin when the cells
    // were kept through the predictor)
    const float reach = K.reach;
    // the CTA's last target: when it lies in the first window's column and
    // rows, that window is the whole CTA and its end needs no further lookup
    // (the usual case; each global round trip here is exposed latency)
    const uint32_t klast = __ldg(F.key + t1 - 1);
    const int cxl = (int)(klast / (uint32_t)ncy);
    const int cyll = (int)klast - cxl * ncy;
    int cur = t0;
    int rows = kTileRows;
    while (cur < t1) {  // block-uniform loop over row windows
        const uint32_t kc = __ldg(F.key + cur);
        const int cx = (int)(kc / (uint32_t)ncy);
        const int cy0 = (int)kc - cx * ncy;
        const int rowlim = min(cy0 + rows, ncy);
        int we, cyl;
        if (cxl == cx && cyll < rowlim) {
            we = t1;
            cyl = cyll;
        } else {
            we = min(t1, (int)__ldg(fstart + cx * ncy + rowlim));
            cyl = (int)__ldg(F.key + we - 1) - cx * ncy;
        }
        const int rlo = max(cy0 - 1, 0), rhi = min(cyl + 1, ncy - 1);
        const int nr = rhi - rlo + 1;
        const int i = cur + tid;
        const bool active = i < we;
        // the target's own cell row, fetched with the cell offsets below
        const uint32_t ki = active ? __ldg(F.key + i) : 0u;
        __syncthreads();  // previous window finished with shared memory
        for (int e = tid; e < 3 * (nr + 1); e += kTileT) {
            const int dxi = e / (nr + 1), q = e - dxi * (nr + 1);
            const int col = cx + dxi - 1;
            int fo = 0, wo = 0;
            if (col >= 0 && col < g.ncx) {
                const int c = col * ncy + rlo + q;
                fo = (int)__ldg(fstart + c);
                wo = (int)__ldg(wstart + c);
            }
            sm.foff[dxi][q] = fo;
            sm.woff[dxi][q] = wo;
        }
        __syncthreads();
        int fb[3], wb[3], f0[3], w0[3];
        int tot = 0, totw = 0;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            w0[d] = sm.woff[d][0];
            f0[d] = sm.foff[d][0];
            wb[d] = tot;
            tot += sm.woff[d][nr] - w0[d];
            totw += sm.woff[d][nr] - w0[d];
            fb[d] = tot;
            tot += sm.foff[d][nr] - f0[d];
        }
        if (tot > SH::cap && rows > 1) {  // too dense: fewer target rows per window
            rows = (rows + 1) >> 1;
            continue;
        }
        Acc4 acc = {0.f, 0.f, 0.f, 0.f};
        float2 la = make_float2(0.f, 0.f), va = make_float2(0.f, 0.f);
        float sa = 0.f, Pa = 0.f, Ia = 0.f, Ra2 = 0.f;
        int cy = 0;
        if (tot <= SH::cap) {
            // ---- stage the neighbour block: slot e of the block is row
            // e - base + first of its segment (walls of column 0, fluid of
            // column 0, walls of column 1, ...); every load of a thread is
            // issued before the first store, one round trip per window.  x is
            // staged relative to the centre column (|x| < 2 kh: the rounding
            // stays at ~1e-7 of a cell), y relative to the particle's own cell
            constexpr int kStage = (SH::cap + kTileT - 1) / kTileT;
            float2 st_l[kStage], st_v[kStage];
            float st_s[kStage], st_p[kStage];
#pragma unroll
            for (int u = 0; u < kStage; u++) {
                const int e = tid + u * kTileT;
                int j = e + w0[0];
                bool wall = true;
                float xs = -khf;  // x of the cell's origin relative to the centre column's
                if (e >= fb[0]) { j = e - fb[0] + f0[0]; wall = false; }
                if (e >= wb[1]) { j = e - wb[1] + w0[1]; wall = true; xs = 0.f; }
                if (e >= fb[1]) { j = e - fb[1] + f0[1]; wall = false; }
                if (e >= wb[2]) { j = e - wb[2] + w0[2]; wall = true; xs = khf; }
                if (e >= fb[2]) { j = e - fb[2] + f0[2]; wall = false; }
                st_l[u] = make_float2(0.f, 0.f);
                st_v[u] = make_float2(0.f, 0.f);
                st_s[u] = 0.f;
                st_p[u] = 0.f;
                if (e < tot) {
                    st_l[u] = __ldg((wall ? Wl.loc : F.loc) + j);
                    st_l[u].x += xs;
                    st_s[u] = __ldg((wall ? Wl.rho : F.rho) + j);
                    if (STORED_P) st_p[u] = __ldg((wall ? Wl.p : F.p) + j);
                    if (!wall) st_v[u] = __ldg(F.v + j);
                }
            }
#pragma unroll
            for (int u = 0; u < kStage; u++) {
                const int e = tid + u * kTileT;
                if (e < tot) {
                    const float s = st_s[u];
                    const float p = STORED_P ? st_p[u] : eos(s, P);
                    const float ib = rcp_approx(P.rho0 + s);
                    sm.loc[e] = st_l[u];
                    sm.vs[e] = staged_vs(st_v[u], s, p, ib);
                    sm.inv[e] = ib;
                }
            }
            __syncthreads();
            if (active) {
                cy = (int)ki - cx * ncy;
                const int own = fb[1] + (i - f0[1]);
                la = sm.loc[own];
                // ---- phase 1: in-support neighbours into the list (entry:
                // staged index << 2 | row code).  Per column the rows below,
                // own and above are staged ranges [R0, R1), [R1, R2), [R2, R3).
                bool overflow = false;
                uint16_t *const lst = sm.list + tid;
                uint16_t *const wend = lst + SH::list * kTileT;
                uint16_t *w = lst;
                const float by_b = la.y + khf, by_a = la.y - khf;
                const int q = cy - rlo;
                const bool hb = cy >= 1, ha = cy + 1 < ncy;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const int col = cx + d - 1;
                    if (col < 0 || col >= g.ncx) continue;
#pragma unroll
                    for (int kind = 0; kind < 2; kind++) {
                        if (kind == 0 && totw == 0) continue;  // block-uniform: no walls here
                        const int *offs = kind == 0 ? sm.woff[d] : sm.foff[d];
                        const int base = kind == 0 ? wb[d] - w0[d] : fb[d] - f0[d];
                        const int R1 = base + offs[q], R2 = base + offs[q + 1];
                        const int R0 = hb ? base + offs[q - 1] : R1;
                        const int R3 = ha ? base + offs[q + 2] : R2;
                        // a range that could overflow the list is skipped (the
                        // target then takes the global-memory path)
                        if (wend - w < (R2 - R1) * kTileT) overflow = true;
                        else if (d == 1 && kind == 1)
                            w = scan_own<kTileT, true>(sm.loc, R1, R2, la.x, la.y, K.four_h2, w);
                        else
                            w = scan_own<kTileT, false>(sm.loc, R1, R2, la.x, la.y, K.four_h2, w);
                        if (wend - w < (R3 - R2) * kTileT) overflow = true;
                        else w = scan_above<kTileT>(sm.loc, R2, R3, la.x, by_a, K.four_h2, reach, w);
                        if (wend - w < (R1 - R0) * kTileT) overflow = true;
                        else w = scan_below<kTileT>(sm.loc, R0, R1, la.x, by_b, K.four_h2, reach, w);
                    }
                }
                const int cnt = (int)((w - lst) / kTileT);
                // the target's own terms (read after phase 1: fewer live registers there)
                const float4 vsa = sm.vs[own];
                va = make_float2(vsa.x, vsa.y);
                sa = vsa.z;
                Pa = vsa.w;
                Ia = sm.inv[own];
                Ra2 = K.two_rho0 + sa;
                if (!overflow) {
                    // ---- phase 2: the pair terms over the list, two at a time
                    int k = 0;
                    for (; k + 1 < cnt; k += 2) {
                        const uint32_t e0 = lst[k * kTileT], e1 = lst[(k + 1) * kTileT];
                        const float oy0 = sm.offy[e0 & 3u], oy1 = sm.offy[e1 & 3u];
                        const int j0 = (int)(e0 >> 2), j1 = (int)(e1 >> 2);
                        const float2 lb0 = sm.loc[j0], lb1 = sm.loc[j1];
                        const float4 b0 = sm.vs[j0], b1 = sm.vs[j1];
                        const float ib0 = sm.inv[j0], ib1 = sm.inv[j1];
                        pair_terms(la.x - lb0.x, (la.y + oy0) - lb0.y, va.x - b0.x,
                                   va.y - b0.y, sa, Pa, Ia, Ra2, b0.z, b0.w, ib0, K, acc);
                        pair_terms(la.x - lb1.x, (la.y + oy1) - lb1.y, va.x - b1.x,
                                   va.y - b1.y, sa, Pa, Ia, Ra2, b1.z, b1.w, ib1, K, acc);
                    }
                    if (k < cnt) {
                        const uint32_t e = lst[k * kTileT];
                        const int j = (int)(e >> 2);
                        const float oy = sm.offy[e & 3u];
                        const float2 lb = sm.loc[j];
                        const float4 b = sm.vs[j];
                        pair_terms(la.x - lb.x, (la.y + oy) - lb.y, va.x - b.x,
                                   va.y - b.y, sa, Pa, Ia, Ra2, b.z, b.w, sm.inv[j], K, acc);
                    }
                } else {
                    target_global<STORED_P>(F, fstart, wstart, Wl, g, P, K, i, cx, cy, la, va, sa,
                                            Pa, Ia, Ra2, acc);
                }
            }
        } else if (active) {
            cy = (int)ki - cx * ncy;
            la = __ldg(F.loc + i);
            va = __ldg(F.v + i);
            sa = __ldg(F.rho + i);
            const float p = STORED_P ? __ldg(F.p + i) : eos(sa, P);
            Ia = rcp_approx(P.rho0 + sa);
            Pa = p * Ia;
            Ra2 = K.two_rho0 + sa;
            target_global<STORED_P>(F, fstart, wstart, Wl, g, P, K, i, cx, cy, la, va, sa, Pa, Ia,
                                    Ra2, acc);
        }
        if (active) {
            const float mb = P.m * P.bwen_h;
            const float ax = acc.ax * mb;
            const float ay = fmaf(acc.ay, mb, -P.g);
            const float drho = mb * fmaf(-P.k_psi, acc.diff, acc.cont);
            if constexpr (MODE == MODE_FORCES) {
                F.a[i] = make_float2(ax, ay);
                F.drho[i] = drho;
            } else {
                // Integrate_SymplecticCorrector (src/SPH_integration.h:289-309):
                // rho from the epsilon form with 1/rho_a already at hand, the
                // displacement (v + v_o) dt/2 in FP32, one FP64 add per axis
                const float so = O.rho[i];
                const float e = -drho * Ia * dt;
                const float ie = rcp_approx(2.f + e);
                const float s_new = so * ((2.f - e) * ie) - P.rho0 * (2.f * e * ie);
                const float2 vo = O.v[i];
                const float2 nv = make_float2(fmaf(ax, dt, vo.x), fmaf(ay, dt, vo.y));
                const float hdt = 0.5f * dt;
                const double2 ro = O.r[i];
                const double2 rn = make_double2(ro.x + (double)((nv.x + vo.x) * hdt),
                                                ro.y + (double)((nv.y + vo.y) * hdt));
                out.r[i] = rn;
                reinterpret_cast<float2 *>(out.v)[i] = nv;
                reinterpret_cast<float *>(out.rho)[i] = s_new;
                uint32_t nk;
                bool listed = false;
                int ncx_, ncy_;
                if (out_of_domain_bits(rn, out.boxb)) {
                    // an erase candidate: its cell kept in case the erase skips it
                    nk = cell_key(g, rn, (uint32_t)(cx * ncy + cy), &ncx_, &ncy_);
                    listed = list_removal(out.rm, i);
                    if (!listed) {
                        nk = (uint32_t)g.ncells;
                        atomicOr(health, kHealthRemoved);
                    }
                } else {
                    nk = cell_key(g, rn, (uint32_t)(cx * ncy + cy), &ncx_, &ncy_);
                    if (nk == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
                }
                if (!(nv.x == nv.x) || !(nv.y == nv.y) || !(s_new == s_new))
                    atomicOr(health, kHealthNan);
                out.key[i] = nk;
                if (!listed) out.slot[i] = atomicAdd(out.counts + nk, 1u);
            }
        }
        cur = we;
        rows = kTileRows;
    }
}

inline TileConst make_tile_const(const Phys<float> &P, double h, double rho0, double g, double cs) {
    TileConst K;
    K.neg_half_inv_h = (float)(-0.5 / h);
    K.eps_h2 = P.eps_h2;
    K.four_h2 = P.four_h2;
    K.k_av = P.k_av;
    const double xg = 7.0 * g / (cs * cs);
    K.c1 = (float)(rho0 * xg / 7.0);
    K.c2 = (float)(-rho0 * 3.0 / 49.0 * xg * xg);
    K.two_rho0 = (float)(2.0 * rho0);
    K.reach = (float)(2.0 * h * 1.0001);
    return K;
}

}  // namespace tsph

namespace tsph {

// mDBC ghost-node density, FP32 build: 4 or 2 lanes per wall particle
// (kMdbcLanes, kMdbcLanesMany below; the fused launch leaves room beside
// its wall blocks for the predictor's),
// the 12 moment sums (src/SPH_kernel_approx.h:1237-1287) in FP32, reduced
// with shuffles; the 3x3 solve in FP64 with one reciprocal of the determinant
// (threshold 0.001 and the Shepard / 1000 fall-backs of :1290-1333), the
// clamp at 1000 of src/SPH_mDBC.h:43-44.
// With `predict` the wall's predictor step follows in the same thread
// (rho_o = rho, rho += drho dt/2, as k_predict_keep does for walls).
// Lanes per wall particle: 4 while the walls fit in about two waves of
// resident threads, 2 beyond (a thread then walks more candidates, but more
// walls are in flight: the sums wait on their candidates' loads).  Measured on
// GB300: 19k walls 17.7 us with 4 lanes (19.7 with 8, 21.2 with 2); 1.2 M
// walls 243 us with 2 (299 with 4, 428 with 8, 270 with 1).
constexpr int kMdbcLanes = 4, kMdbcLanesMany = 2;
inline int mdbc_lanes(long long nw, int sms) {
    return nw * kMdbcLanes > 2LL * sms * 4 * kBlock ? kMdbcLanesMany : kMdbcLanes;
}

// the ghost node's 3x3 moment system of one wall (its 12 FP32 sums) solved
// in FP64, the density extrapolated to the wall particle and clamped, then
// the wall's predictor step when `predict`
__device__ __forceinline__ void solve_mdbc(int w, const float *s, const WallState<float> &Wl,
                                           const Phys<float> &P, bool predict, float dt,
                                           const PairRec &RW) {
    // The reference solves A x = (sum m W, sum m dr_x F, sum m dr_y F) for
    // x = (rho, grad rho).  With m = V_b rho_b and A's first column
    // (sum V W, sum V dr_x F, sum V dr_y F), the same system with the
    // right-hand side sum V (rho_b - rho0) (W, dr_x F, dr_y F) has the
    // solution (rho - rho0, grad rho): identical in exact arithmetic, ~1000x
    // smaller numbers (and rounding errors) in FP32.
    const double rhoWsum = s[0], drhodx = s[1], drhody = s[2];
    const double a11 = s[3], a12 = s[4], a13 = s[5], a21 = s[6], a22 = s[7], a23 = s[8],
                 a31 = s[9], a32 = s[10], a33 = s[11];
    const double det = det3(a11, a12, a13, a21, a22, a23, a31, a32, a33);
    double dens;
    if (det > 0.001) {
        const double id = 1.0 / det;
        const double i11 = (a22 * a33 - a23 * a32) * id;
        const double i12 = -(a12 * a33 - a13 * a32) * id;
        const double i13 = (a12 * a23 - a13 * a22) * id;
        const double i21 = -(a21 * a33 - a23 * a31) * id;
        const double i22 = (a11 * a33 - a13 * a31) * id;
        const double i23 = -(a11 * a23 - a13 * a21) * id;
        const double i31 = (a21 * a32 - a22 * a31) * id;
        const double i32 = -(a11 * a32 - a12 * a31) * id;
        const double i33 = (a11 * a22 - a12 * a21) * id;
        const double dens_temp = rhoWsum * i11 + drhodx * i12 + drhody * i13;
        const double grx = -(rhoWsum * i21 + drhodx * i22 + drhody * i23);
        const double gry = -(rhoWsum * i31 + drhodx * i32 + drhody * i33);
        const float2 gnd = Wl.gnd[w];
        dens = dens_temp + grx * (double)gnd.x + gry * (double)gnd.y;  // rho - rho0
    } else if (a11 > 0) {
        dens = rhoWsum / a11;  // Shepard, shifted
    } else {
        dens = 1000. - (double)P.rho0;
    }
    if (dens + (double)P.rho0 < 1000.) dens = 1000. - (double)P.rho0;  // clamp of src/SPH_mDBC.h:44
    const float rw = (float)dens;
    if (predict) {
        Wl.rho_o[w] = rw;
        const float rp = rw + Wl.drho[w] * dt * 0.5f;
        Wl.rho[w] = rp;
        if (RW.v) wall_record(RW, w, rp, P);
    } else {
        Wl.rho[w] = rw;
    }
}

template <int LANES>
__device__ __forceinline__ void mdbc_wall(int gid, const WallState<float> &Wl, int nw,
                                           const uint32_t *__restrict__ fstart,
                                           const FluidState<float> &F, const Grid &g,
                                           const Phys<float> &P, bool predict, float dt,
                                           const PairRec &RW) {
    const int w = gid / LANES, sub = gid % LANES;
    const bool valid = w < nw;
    float s[12];
#pragma unroll
    for (int q = 0; q < 12; q++) s[q] = 0.f;
    const uint32_t gk = valid ? __ldg(Wl.gkey + w) : (uint32_t)g.ncells;
    if (gk < (uint32_t)g.ncells) {
        const int cx = (int)(gk / (uint32_t)g.ncy);
        const int cy = (int)gk - cx * g.ncy;
        const float2 gl = __ldg(Wl.gloc + w);
        // the three rows of a column are contiguous in the sorted state: one
        // candidate range per column, the three fetched together and walked
        // as one list, kUnroll candidates (all their loads) per iteration
        const int ylo = max(cy - 1, 0), yhi = min(cy + 1, g.ncy - 1);
        int jlo[3], n[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const int col = cx + d - 1;
            jlo[d] = 0;
            n[d] = 0;
            if (col >= 0 && col < g.ncx) {
                const int c0 = col * g.ncy;
                jlo[d] = (int)__ldg(fstart + c0 + ylo);
                n[d] = (int)__ldg(fstart + c0 + yhi + 1) - jlo[d];
            }
        }
        const int n01 = n[0] + n[1], ntot = n01 + n[2];
        constexpr int kUnroll = 4;
        for (int e0 = sub; e0 < ntot; e0 += kUnroll * LANES) {
            uint32_t kb[kUnroll];
            float2 lb[kUnroll];
            float sbv[kUnroll];
            int dd[kUnroll];
            bool use[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; u++) {
                const int e = e0 + u * LANES;
                int d = 2, j = jlo[2] + e - n01;
                if (e < n[0]) {
                    d = 0;
                    j = jlo[0] + e;
                } else if (e < n01) {
                    d = 1;
                    j = jlo[1] + e - n[0];
                }
                dd[u] = d;
                use[u] = e < ntot;
                kb[u] = 0u;
                lb[u] = make_float2(0.f, 0.f);
                sbv[u] = 0.f;
                if (use[u]) {
                    kb[u] = __ldg(F.key + j);
                    lb[u] = __ldg(F.loc + j);
                    sbv[u] = __ldg(F.rho + j);
                    if (F.type && __ldg(F.type + j) != 0) use[u] = false;  // fluid only (buffer zones)
                }
            }
#pragma unroll
            for (int u = 0; u < kUnroll; u++) {
                if (!use[u]) continue;
                const int col = cx + dd[u] - 1;
                const int rowb = (int)kb[u] - col * g.ncy;
                const float drx = (gl.x + (float)(1 - dd[u]) * g.khf) - lb[u].x;
                const float dry = (gl.y + (float)(cy - rowb) * g.khf) - lb[u].y;
                const float r2 = fmaf(drx, drx, dry * dry);
                if (!(r2 <= P.four_h2)) continue;
                float W, Fk;
                if (r2 == 0.f) {
                    W = P.awen;
                    Fk = 0.f;
                } else {
                    wendland32(r2, P, W, Fk, true);
                }
                const float sb = sbv[u];  // rho_b - rho0
                const float V = P.m * rcp_approx(P.rho0 + sb);
                const float WV = W * V, FV = Fk * V;
                // right-hand side of the density field shifted by rho0
                s[0] = fmaf(WV, sb, s[0]);
                s[1] = fmaf(drx * FV, sb, s[1]);
                s[2] = fmaf(dry * FV, sb, s[2]);
                s[3] += WV;
                s[4] = fmaf(drx, WV, s[4]);
                s[5] = fmaf(dry, WV, s[5]);
                s[6] = fmaf(drx, FV, s[6]);
                s[7] = fmaf(drx * drx, FV, s[7]);
                s[8] = fmaf(drx * dry, FV, s[8]);
                s[9] = fmaf(dry, FV, s[9]);
                s[10] = fmaf(dry * drx, FV, s[10]);
                s[11] = fmaf(dry * dry, FV, s[11]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 12; q++) {
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    }
    // The FP64 solve runs one wall per lane: GB300 issues FP64 at a small
    // fraction of the FP32 rate and a warp instruction costs the same with 4
    // lanes active as with 32, so the block's 32 walls hand their sums to its
    // first warp (lane l solves wall l of the block) instead of solving in
    // lane 0 of each group of 8.
    constexpr int kWallsPerBlock = kBlock / LANES;
    __shared__ float sums[12][kWallsPerBlock + 1];
    const int wl = (int)threadIdx.x / LANES;
#pragma unroll
    for (int q = 0; q < 12; q++)
        if (q % LANES == sub) sums[q][wl] = s[q];
    __syncthreads();
    if (threadIdx.x >= kWallsPerBlock) return;
    const int ws = gid / kBlock * kWallsPerBlock + (int)threadIdx.x;
    if (ws >= nw) return;
#pragma unroll
    for (int q = 0; q < 12; q++) s[q] = sums[q][threadIdx.x];
    solve_mdbc(ws, s, Wl, P, predict, dt, RW);
}

template <int LANES>
static __global__ void __launch_bounds__(kBlock)
k_mdbc_f32(WallState<float> Wl, int nw, const uint32_t *__restrict__ fstart, FluidState<float> F,
            Grid g, Phys<float> P) {
    pdl_enter();
    mdbc_wall<LANES>(blockIdx.x * blockDim.x + threadIdx.x, Wl, nw, fstart, F, g, P, false, 0.f,
              PairRec{});
}

// fluid particles per thread of the fused predictor
constexpr int kPredU = 4;

// mDBC and the predictor of a step in one launch: the first nbm blocks
// compute the walls' densities (each wall then takes its predictor step),
// the rest run the fluid predictor in the current cell order.  The two halves
// touch disjoint data (mDBC reads F's type, key, loc and rho and writes the
// walls; the fluid predictor reads F and writes D and O), so the
// latency-bound ghost-node sums overlap the bandwidth-bound predictor.
template <int LANES>
static __global__ void __launch_bounds__(kBlock, 4)
k_mdbc_f32_predict(WallState<float> Wl, int nw, int nbm, const uint32_t *__restrict__ fstart,
                FluidState<float> F, Grid g, Phys<float> P, float dt, FluidState<float> D,
                OldState<float> O, float skin, uint32_t *__restrict__ rebuild,
                uint32_t *__restrict__ health, cudaGraphConditionalHandle cond, int use_cond,
                KeepCells kc, PairRec RS, PairRec RW, int interleave) {
    pdl_enter();
    // The block's half: mDBC blocks first (their one wave runs ahead of the
    // predictor's blocks), or, when the walls need several waves
    // (`interleave`), mDBC and predictor blocks alternating, so that the
    // latency-bound ghost-node sums share every wave with the bandwidth-bound
    // predictor
    const int b = (int)blockIdx.x, nbp = (int)gridDim.x - nbm;
    int bm = -1, bp = -1;
    if (interleave) {
        const int pairs = min(nbm, nbp);
        if (b < 2 * pairs) {
            if (b & 1) bp = b >> 1;
            else bm = b >> 1;
        } else if (nbm > pairs) {
            bm = b - pairs;
        } else {
            bp = b - pairs;
        }
    } else if (b < nbm) {
        bm = b;
    } else {
        bp = b - nbm;
    }
    if (bm >= 0) {
        mdbc_wall<LANES>(bm * blockDim.x + threadIdx.x, Wl, nw, fstart, F, g, P, true, dt, RW);
        return;
    }
    predict_keep_fluid_f32<kPredU>(bp * blockDim.x + threadIdx.x, nbp * blockDim.x, F, fstart, g,
                                   dt, D, O, skin, rebuild, health, cond, use_cond, kc, RS, P);
}

}  // namespace tsph
