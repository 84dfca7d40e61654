// tsph_pairs_rec.cuh -- the FP32 pair loop of Compute_Forces
// (src/SPH_interaction.h:8-149, fused with Integrate_SymplecticCorrector,
// src/SPH_integration.h:289-309) over pair records staged by bulk copies.
//
// Pair records.  Before a pair pass, every particle's neighbour-side values
// are formed once, in the sorted order, by k_pair_records (two arrays of
// 16-byte records, so a window's records are a few contiguous ranges of each,
// and a neighbour is two 128-bit shared-memory loads):
//   re[i] = {x relative to the particle's own cell, y relative to that cell,
//            cell row as a float, 1/rho}
//   rv[i] = {vx, vy, rho - rho0, p/rho}
// The support test and the window search use a coarse y in the grid's frame,
// fmaf(row, kh, y) (~1e-7 m rounding: it can only move pairs within ~1e-4 h
// of r = 2h, where W and dW vanish to ~1e-12 of their scale); the pair terms
// form dy from the cell-relative y and the exact row difference, and dx from
// the cell-relative x and the column offset, as precisely as k_pairs_tiled.
//
// Work decomposition: a CTA takes 128 consecutive fluid targets (one thread
// each) and walks them in windows of at most kRecRows rows of one column.
// Per window one thread issues cp.async.bulk copies (1-D TMA) of the
// 3 x (rows + 2) neighbour cells' record ranges (walls and fluid of the three
// columns; each range widened to 4-record alignment) into shared memory,
// completing on an mbarrier: no per-neighbour instructions, one round trip.
// Phase 1 walks, per neighbour column, one contiguous y-window of the
// y-sorted column (both ends by binary search on the coarse y), so every lane
// of a warp runs about the same number of candidates, and keeps the
// in-support neighbours in a per-thread list of (staged index, column)
// entries; a segment is scanned in pieces of at most a list's capacity, and
// when a piece might not fit in some lane's list the whole warp sums its lists
// (phase 2) and empties them first (a warp-uniform step, so no lane waits on
// another's): the pairs are still summed in candidate order.  Phase 2 sums the WCSPH pair terms (pair_terms
// of k_pairs_tiled) over the list.
//
// With the cells of the last binning kept through the predictor the columns
// are y-sorted as of that binning and every particle has moved less than the
// skin since: K.reach includes twice the skin (and the coarse y's rounding),
// which keeps the search and the early stop conservative.
#pragma once

#include "tsph_pairs_tiled.cuh"

namespace tsph {

constexpr int kRecT = 128;    // targets per CTA (one thread each)
constexpr int kRecRows = 16;  // max target rows per window
constexpr int kRecPad = 1;    // records per 16 bytes (every record array is 16 B wide)

constexpr unsigned long long kWaitNs = 4000000000ull;  // bounded mbarrier waits (4 s)
constexpr int kRecMaxWin = 4;  // windows per chunk in the window table
constexpr int kRecOffRun = ((kRecRows + 3 + 3) + 3) & ~3;  // offsets copied per column
enum { kRecStaged = 0, kRecGlobal = 1 };

// One window of a chunk (written by k_pair_records, read by k_pairs_rec):
// targets [cur, we) in rows rlo+1.. of column cx, staged rows [rlo, rlo+nr);
// segment s (walls, fluid of columns cx-1, cx, cx+1) is staged from global
// row first[s], n[s] rows.  lrows: the entries of the longest stored list of
// the window's targets (set by the pass that builds the lists; -1: not known,
// the whole list block), the rows of the list block a later pass copies.
struct __align__(16) WinRec {
    int cur, we, cx, rlo, nr, mode, tot, lrows;
    int first[6];
    int n[6];
};

template <int CAP, int LIST> struct RecShape {
    static constexpr int cap = CAP, list = LIST;
};
typedef RecShape<528, 38> RecStd;


// Neighbour lists kept between passes (the fused step).  A pass right after
// a binning (positions exactly as binned) builds every target's list of the
// neighbours within 2h + 2 sigma and stores it; later passes, while every
// particle stays within sigma of where it was binned, sum the stored lists
// (the kernel factor clamped at zero beyond 2h) with no candidate search.
// A pass builds when the count of sorts (gen[0], bumped by every sort)
// differs from the sort the lists were built after (gen[1], set by the last
// CTA of every pass).
// Cases packed into one system (the batched workload): every case scaled to
// the system's particle spacing, so that all SPH constants but gravity (and
// the two Fourtakas coefficients that follow from it) are shared; each case
// keeps its own removal box.  A grid column belongs to one case.
struct CaseConst {
    float g, c1, c2, pad;
    BoxBits box;
};

struct RecStep {
    uint16_t *glist;            // [chunk][list][128]: entries (staged index << 2 | column)
    uint8_t *gcnt;              // [chunk][128]: entries, or 255 (did not fit: global path)
    uint32_t *gen;              // {sorts, sort the lists were built after, -, CTAs done}
    const float2 *lbin;         // cell-relative positions at the binning
    float sig2;                 // squared displacement allowed since the binning
    // MODE_CORRECT: the new state is written in the kept order (out.r, out.v,
    // out.rho are the current buffers); these take its cell-relative
    // positions and the pair records of the next pass
    float2 *nloc;
    PairRec nrec;
    uint32_t *need_sort;        // MODE_CORRECT: set when the cells must be rebuilt
    cudaGraphConditionalHandle cond_sort;
    int use_cond;
    // packed cases (kernels instantiated with CASES): the case of each grid
    // column and each case's constants
    const int32_t *col_case = nullptr;
    const CaseConst *cases = nullptr;
};

template <class SH> struct RecSmem {
    float4 e[SH::cap];
    float4 v[SH::cap];
    uint16_t list[SH::list * kRecT];
    // fstart / wstart of the staged rows of each column, copied from the
    // 4-aligned index below (col * ncy + rlo); row q of column d is at
    // [d][q + oshift[d]]
    int foff[3][kRecOffRun];
    int woff[3][kRecOffRun];
    int oshift[3];
    int base[6];  // staged index of global row j of segment s = base[s] + j
    WinRec win;
    __align__(16) uint8_t cnt[kRecT];  // stored list lengths of the chunk's targets
    unsigned long long bar;
    // the window's case (kernels with CASES) and its pair constants
    TileConst kc;
    int kcase;
    int lmax;  // the longest list stored in this window (a pass that builds them)
};


// ---------------------------------------------------------------- records
// The windows of chunk c (targets [128 c, 128 c + 128) of the live rows): at
// most kRecRows target rows of one column each, halved while the staged
// block exceeds `cap`; a block that does not fit even for one row, and the
// rest of a chunk that needs more than kRecMaxWin windows, take the
// global-memory path.
__device__ __forceinline__ void rec_window_table(int c, int cap, const FluidState<float> &F,
                                                 const uint32_t *__restrict__ fstart,
                                                 const uint32_t *__restrict__ wstart,
                                                 const Grid &g, WinRec *__restrict__ table,
                                                 int *__restrict__ nwin) {
    const int nl = n_live(fstart, g.ncells);
    const int t0 = c * kRecT;
    if (t0 >= nl) {
        nwin[c] = 0;
        return;
    }
    const int ncy = g.ncy;
    const int t1 = min(t0 + kRecT, nl);
    const uint32_t klast = __ldg(F.key + t1 - 1);
    const int cxl = (int)(klast / (uint32_t)ncy);
    const int cyll = (int)klast - cxl * ncy;
    int cur = t0, nwc = 0;
    while (cur < t1 && nwc < kRecMaxWin) {
        const uint32_t kc = __ldg(F.key + cur);
        const int cx = (int)(kc / (uint32_t)ncy);
        const int cy0 = (int)kc - cx * ncy;
        WinRec R;
        int rows = kRecRows, we, tot;
        for (;;) {
            const int rowlim = min(cy0 + rows, ncy);
            int cyl;
            if (cxl == cx && cyll < rowlim) {
                we = t1;
                cyl = cyll;
            } else {
                we = min(t1, (int)__ldg(fstart + cx * ncy + rowlim));
                cyl = (int)__ldg(F.key + we - 1) - cx * ncy;
            }
            R.rlo = max(cy0 - 1, 0);
            const int rhi = min(cyl + 1, ncy - 1);
            R.nr = rhi - R.rlo + 1;
            tot = 0;
            for (int sgi = 0; sgi < 6; sgi++) {
                const int col = cx + (sgi >> 1) - 1;
                const uint32_t *st = (sgi & 1) ? fstart : wstart;
                int j0 = 0, j1 = 0;
                if (col >= 0 && col < g.ncx) {
                    j0 = (int)__ldg(st + col * ncy + R.rlo);
                    j1 = (int)__ldg(st + col * ncy + rhi + 1);
                }
                const int a0 = j0 & ~(kRecPad - 1);
                const int cnt = j1 > j0 ? ((j1 - a0 + kRecPad - 1) & ~(kRecPad - 1)) : 0;
                R.first[sgi] = a0;
                R.n[sgi] = cnt;
                tot += cnt;
            }
            if (tot > cap && rows > 1) {
                rows = (rows + 1) >> 1;
                continue;
            }
            break;
        }
        R.mode = tot <= cap ? kRecStaged : kRecGlobal;
        if (nwc == kRecMaxWin - 1 && we < t1) {
            we = t1;
            R.mode = kRecGlobal;
        }
        R.cur = cur;
        R.we = we;
        R.cx = cx;
        R.tot = tot;
        R.lrows = -1;
        table[(size_t)c * kRecMaxWin + nwc] = R;
        nwc++;
        cur = we;
    }
    nwin[c] = nwc;
}

// pair records of the fluid rows [0, n_live) and the walls [0, nw) of a state
// (p from the EOS of rho, or the stored p); the blocks from `rec_blocks` on
// build the window table, one thread per chunk of 128 targets, when the
// coming pass builds the lists
template <bool STORED_P>
__global__ void __launch_bounds__(kBlock)
k_pair_records(FluidState<float> F, const uint32_t *__restrict__ fstart, WallState<float> Wl,
               int nw, Grid g, Phys<float> P, PairRec RF, PairRec RW, int rec_blocks,
               const uint32_t *__restrict__ wstart, int nchunks, int cap,
               WinRec *__restrict__ table, int *__restrict__ nwin, uint32_t *__restrict__ gen,
               const uint32_t *__restrict__ gate, int force_table) {
    pdl_enter();
    if (gated_off(gate)) return;
    if ((int)blockIdx.x >= rec_blocks) {
        // the table follows the cells: rebuilt after a sort (the lists are
        // then stale until a pass builds them), or on request
        const int c = ((int)blockIdx.x - rec_blocks) * blockDim.x + threadIdx.x;
        if (c < nchunks && (force_table || __ldg(gen) != __ldg(gen + 1)))
            rec_window_table(c, cap, F, fstart, wstart, g, table, nwin);
        return;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nl = n_live(fstart, g.ncells);
    const bool wall = i < nw;
    const int j = wall ? i : i - nw;
    if (!wall && j >= nl) return;
    const uint32_t key = __ldg((wall ? Wl.key : F.key) + j);
    const float2 l = __ldg((wall ? Wl.loc : F.loc) + j);
    const float s = __ldg((wall ? Wl.rho : F.rho) + j);
    const float2 v = wall ? make_float2(0.f, 0.f) : __ldg(F.v + j);
    const float p = STORED_P ? __ldg((wall ? Wl.p : F.p) + j) : eos(s, P);
    const int cx = (int)(key / (uint32_t)g.ncy);
    const float row = (float)((int)key - cx * g.ncy);
    const float ib = rcp_approx(P.rho0 + s);
    (wall ? RW.e : RF.e)[j] = make_float4(l.x, l.y, row, ib);
    (wall ? RW.v : RF.v)[j] = make_float4(v.x, v.y, s, p * ib);
}

// ---------------------------------------------------------------- plumbing
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(
                     smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0u;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// wait for the phase with the given parity to complete; false after
// kWaitNs (the caller then records kHealthStall and leaves)
__device__ __forceinline__ bool mbar_wait(unsigned long long *b, uint32_t parity) {
    if (mbar_try(b, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try(b, parity))
        if (global_ns() - t0 > kWaitNs) return false;
    return true;
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         unsigned long long *b) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(b))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// the coarse y of a record in the grid's frame (support test and search)
__device__ __forceinline__ float rec_ycoarse(const float4 &r, float khf) {
    return fmaf(r.z, khf, r.y);
}

// phase 1 over candidates [s, e) of one segment: entry = staged index << 2 |
// column for every candidate within the test radius (h2 = its square);
// `excl` (the target's own column) also drops r = 0, the target itself
__device__ __forceinline__ uint16_t *rec_scan(const float4 *__restrict__ t, int s, int e, float xa,
                                              float ya, float khf, float h2, bool excl,
                                              uint32_t col, uint16_t *w) {
    const float lo2 = excl ? 0.f : -1.f;  // kept when lo2 < r2 <= h2
    int j = s;
    uint32_t ent = ((uint32_t)s << 2) | col;
    for (; j + 1 < e; j += 2, ent += 8u) {
        const float4 l0 = t[j], l1 = t[j + 1];
        const float dx0 = xa - l0.x, dy0 = ya - rec_ycoarse(l0, khf);
        const float dx1 = xa - l1.x, dy1 = ya - rec_ycoarse(l1, khf);
        const float r0 = fmaf(dx0, dx0, dy0 * dy0), r1 = fmaf(dx1, dx1, dy1 * dy1);
        *w = (uint16_t)ent;
        w += (r0 <= h2 && r0 > lo2) ? kRecT : 0;
        *w = (uint16_t)(ent + 4u);
        w += (r1 <= h2 && r1 > lo2) ? kRecT : 0;
    }
    if (j < e) {
        const float4 l = t[j];
        const float dx = xa - l.x, dy = ya - rec_ycoarse(l, khf);
        const float r = fmaf(dx, dx, dy * dy);
        *w = (uint16_t)ent;
        w += (r <= h2 && r > lo2) ? kRecT : 0;
    }
    return w;
}

// first index of [lo, hi) whose coarse y is not below y (ABOVE: above y)
template <bool ABOVE>
__device__ __forceinline__ int rec_bound(const float4 *__restrict__ t, int lo, int hi, float y,
                                         float khf) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const float ym = rec_ycoarse(t[mid], khf);
        if (ABOVE ? !(ym > y) : (ym < y)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// phase 2: the pair terms over list entries [0, cnt)
// the target's x in the frame of neighbour column code c (0, 1, 2: the
// column right of, at, left of the target's), by selects instead of a
// shared-memory table
__device__ __forceinline__ float rec_xcol(uint32_t c, float xp, float x0, float xm) {
    return (c & 2u) ? xm : ((c & 1u) ? x0 : xp);
}

template <class SH>
__device__ __forceinline__ void rec_eval(const RecSmem<SH> &sm, const uint16_t *lst, int cnt,
                                         float xa, float yca, float rowa, float2 va, float sa,
                                         float Pa, float Ia, float Ra2, float khf,
                                         const TileConst &K, Acc4 &acc) {
    const float xp = xa + khf, xm = xa - khf;
    int k = 0;
    for (; k + 1 < cnt; k += 2) {
        const uint32_t e0 = lst[k * kRecT], e1 = lst[(k + 1) * kRecT];
        const int j0 = (int)(e0 >> 2), j1 = (int)(e1 >> 2);
        const float4 a0 = sm.e[j0], a1 = sm.e[j1];
        const float4 v0 = sm.v[j0], v1 = sm.v[j1];
        pair_terms<true>(rec_xcol(e0, xp, xa, xm) - a0.x, fmaf(rowa - a0.z, khf, yca - a0.y),
                         va.x - v0.x, va.y - v0.y, sa, Pa, Ia, Ra2, v0.z, v0.w, a0.w, K, acc);
        pair_terms<true>(rec_xcol(e1, xp, xa, xm) - a1.x, fmaf(rowa - a1.z, khf, yca - a1.y),
                         va.x - v1.x, va.y - v1.y, sa, Pa, Ia, Ra2, v1.z, v1.w, a1.w, K, acc);
    }
    if (k < cnt) {
        const uint32_t e = lst[k * kRecT];
        const int j = (int)(e >> 2);
        const float4 a = sm.e[j];
        const float4 v = sm.v[j];
        pair_terms<true>(rec_xcol(e, xp, xa, xm) - a.x, fmaf(rowa - a.z, khf, yca - a.y),
                         va.x - v.x, va.y - v.y, sa, Pa, Ia, Ra2, v.z, v.w, a.w, K, acc);
    }
}

// store a target's current list segment [0, cnt) after the entries already
// stored (gpos), or mark the list as too long
__device__ __forceinline__ void rec_store(uint16_t *__restrict__ gl, const uint16_t *lst, int cnt,
                                          int cap, int &gpos, bool &over) {
    if (over) return;
    if (gpos + cnt > cap) {
        over = true;
        return;
    }
    for (int k = 0; k < cnt; k++) gl[(size_t)(gpos + k) * kRecT] = lst[k * kRecT];
    gpos += cnt;
}

template <int MODE, bool STORED_P, class SH, bool CASES = false>
__global__ void __launch_bounds__(kRecT, 8)
k_pairs_rec(FluidState<float> F, const uint32_t *__restrict__ fstart,
            const uint32_t *__restrict__ wstart, WallState<float> Wl, Grid g, Phys<float> P,
            TileConst K, TileConst Kb, OldState<float> O, float dt, PairOut out, PairRec RF,
            PairRec RW, const WinRec *__restrict__ table, const int *__restrict__ nwin,
            RecStep S, uint32_t *__restrict__ health) {
    __shared__ __align__(16) RecSmem<SH> sm;
    pdl_enter();
    const int tid = threadIdx.x;
    const int ncy = g.ncy;
    const float khf = g.khf;
    const int nw = __ldg(nwin + blockIdx.x);
    // this pass builds and stores the lists when a sort happened since they
    // were built (the last CTA to finish records the sort they are built after)
    const bool build = MODE == MODE_LISTS || __ldg(S.gen) != __ldg(S.gen + 1);
    auto finish = [&]() {
        if (tid == 0) {
            __threadfence();
            if (atomicAdd(S.gen + 3, 1u) == gridDim.x - 1) {
                S.gen[1] = S.gen[0];
                S.gen[3] = 0u;
                __threadfence();
            }
        }
    };
    const int t0 = blockIdx.x * kRecT;
    // the chunk's stored lists: column (i - t0) of a [list][128] block
    uint16_t *const gblock = S.glist + (size_t)blockIdx.x * SH::list * kRecT;
    if (tid == 0) {
        mbar_init(&sm.bar, 1);
        fence_mbar_init();
    }
    uint32_t parity = 0u;
    // a pass that builds the lists records, per window, its longest list
    WinRec *const table_w = const_cast<WinRec *>(table) + (size_t)blockIdx.x * kRecMaxWin;
    for (int wi = 0; wi < nw; wi++) {
        __syncthreads();  // the previous window is finished with shared memory
        if (tid == 0) {
            if (build && wi > 0) table_w[wi - 1].lrows = sm.lmax;
            sm.lmax = 0;
            // the window's record, then one bulk copy per record array and
            // segment, per offset run (lists built here) or of the chunk's
            // stored lists (lists kept), all completing on the mbarrier
            const WinRec R = table[(size_t)blockIdx.x * kRecMaxWin + wi];
            sm.win = R;
            if constexpr (CASES) {
                const CaseConst C = S.cases[__ldg(S.col_case + R.cx)];
                sm.kc = K;
                sm.kc.c1 = C.c1;
                sm.kc.c2 = C.c2;
                sm.kcase = __ldg(S.col_case + R.cx);
            }
            if (R.mode == kRecStaged) {
                uint32_t bytes = (uint32_t)R.tot * 32u;
                int at = 0;
                for (int sgi = 0; sgi < 6; sgi++) {
                    sm.base[sgi] = at - R.first[sgi];
                    at += R.n[sgi];
                }
                const bool lists = !build;
                if (build) {
                    for (int d = 0; d < 3; d++) {
                        const int col = R.cx + d - 1;
                        if (col >= 0 && col < g.ncx) bytes += 2u * 4u * (uint32_t)kRecOffRun;
                    }
                }
                const int lr = R.lrows < 0 ? SH::list : R.lrows;  // list rows to copy
                if (lists) bytes += (uint32_t)(lr * kRecT * 2 + kRecT);
                fence_proxy_async_smem();  // the previous window's reads before the copies
                mbar_expect_tx(&sm.bar, bytes);
                at = 0;
                for (int sgi = 0; sgi < 6; sgi++) {
                    const int c = R.n[sgi];
                    if (c > 0) {
                        const bool fl = sgi & 1;
                        const int j = R.first[sgi];
                        bulk_g2s(&sm.e[at], (fl ? RF.e : RW.e) + j, (uint32_t)c * 16u, &sm.bar);
                        bulk_g2s(&sm.v[at], (fl ? RF.v : RW.v) + j, (uint32_t)c * 16u, &sm.bar);
                    }
                    at += c;
                }
                if (build) {
                    for (int d = 0; d < 3; d++) {
                        const int col = R.cx + d - 1;
                        if (col >= 0 && col < g.ncx) {
                            const int so = col * ncy + R.rlo, sa = so & ~3;
                            sm.oshift[d] = so - sa;
                            bulk_g2s(&sm.foff[d][0], fstart + sa, 4u * kRecOffRun, &sm.bar);
                            bulk_g2s(&sm.woff[d][0], wstart + sa, 4u * kRecOffRun, &sm.bar);
                        }
                    }
                }
                if (lists) {
                    if (lr > 0) bulk_g2s(sm.list, gblock, (uint32_t)(lr * kRecT * 2), &sm.bar);
                    bulk_g2s(sm.cnt, S.gcnt + t0, (uint32_t)kRecT, &sm.bar);
                }
            }
        }
        __syncthreads();  // the window's record is visible
        const int cur = sm.win.cur, we = sm.win.we, cx = sm.win.cx, rlo = sm.win.rlo;
        // the window's pair constants: the system's, with the case's two
        // gravity-dependent coefficients in registers (kernels with CASES)
        TileConst Kw = K;
        if constexpr (CASES) {
            Kw.c1 = sm.kc.c1;
            Kw.c2 = sm.kc.c2;
        }
        const int mode = sm.win.mode;
        const int i = cur + tid;
        const bool active = i < we;
        const int col_i = i - t0;  // the target's column of the chunk's lists
        // the corrector's old state and binning position, fetched while the
        // window is staged
        double2 ro_r = make_double2(0., 0.);
        float2 ro_v = make_float2(0.f, 0.f), lb = make_float2(0.f, 0.f);
        float ro_s = 0.f;
        if (MODE == MODE_CORRECT && active) {
            ro_r = O.r[i];
            ro_v = O.v[i];
            ro_s = O.rho[i];
            lb = S.lbin[i];
        }
        Acc4 acc = {0.f, 0.f, 0.f, 0.f};
        float Ia = 0.f;
        int cxa = cx, cy = 0;
        bool global = mode != kRecStaged;
        int tcase = 0;  // the target's case (kernels with CASES)
        if constexpr (CASES) tcase = sm.kcase;
        const unsigned amask = __ballot_sync(0xffffffffu, active);  // the warp's targets
        if (mode == kRecStaged) {
            const bool ok = mbar_wait(&sm.bar, parity);
            parity ^= 1u;
            if (!ok) {
                // the copies did not complete in time: record it, give them one
                // more bounded wait, and leave without touching the window
                if (tid == 0) atomicOr(health, kHealthStall);
                mbar_wait(&sm.bar, parity ^ 1u);
                finish();
                return;
            }
            const bool walls = (sm.win.n[0] | sm.win.n[2] | sm.win.n[4]) != 0;
            if (active) {
                const int own = sm.base[3] + i;
                const float4 ae = sm.e[own];
                const float4 av = sm.v[own];
                Ia = ae.w;
                const float xa = ae.x, ya = rec_ycoarse(ae, khf), yca = ae.y, rowa = ae.z;
                cy = (int)rowa;
                const float2 va = make_float2(av.x, av.y);
                const float sa = av.z, Pa = av.w, Ra2 = K.two_rho0 + sa;
                uint16_t *const lst = sm.list + col_i;
                if (!build) {
                    // the stored list (built after the last binning)
                    const int c = (int)sm.cnt[col_i];
                    if (c == 255) global = true;
                    else if (MODE != MODE_LISTS)
                        rec_eval(sm, lst, c, xa, yca, rowa, va, sa, Pa, Ia, Ra2, khf,
                                 Kw, acc);
                } else {
                    // phase 1 at radius Kb (2h + 2 sigma), the list stored
                    // segment by segment as it is summed
                    const float ybot = ya - Kb.reach, ytop = ya + Kb.reach;
                    uint16_t *const wend = lst + SH::list * kRecT;
                    uint16_t *w = lst;
                    uint16_t *const gl = gblock + col_i;
                    int gpos = 0;
                    bool over = false;
                    const int q = cy - rlo;
                    const int qlo = cy >= 1 ? q - 1 : q, qhi = cy + 1 < ncy ? q + 2 : q + 1;
                    // the six segments in staged order: walls (scanned whole)
                    // and fluid (over its y-window) of the three columns
#pragma unroll 1
                    for (int sgi = walls ? 0 : 1; sgi < 6; sgi += walls ? 1 : 2) {
                        const int d = sgi >> 1;
                        const int col = cx + d - 1;
                        if (col < 0 || col >= g.ncx) continue;
                        const float xd = xa + (float)(1 - d) * khf;  // the target's x in column d's frame
                        const int osh = sm.oshift[d];
                        const int bs = sm.base[sgi];
                        int lo, e;
                        if (sgi & 1) {
                            const int re = bs + sm.foff[d][qhi + osh];
                            lo = rec_bound<false>(sm.e, bs + sm.foff[d][qlo + osh], re, ybot, khf);
                            e = rec_bound<true>(sm.e, lo, re, ytop, khf);
                        } else {
                            lo = bs + sm.woff[d][qlo + osh];
                            e = bs + sm.woff[d][qhi + osh];
                        }
                        // pieces of at most a list's capacity; before a piece
                        // that might not fit in some lane's list, the whole warp
                        // sums and empties its lists (the warp runs as many
                        // pieces as its longest segment needs)
                        const int np =
                            (int)__reduce_max_sync(amask, (unsigned)((e - lo + SH::list - 1) / SH::list));
                        for (int pc = 0; pc < np; pc++) {
                            const int pl = min(e, lo + pc * SH::list);
                            const int pe = min(e, pl + SH::list);
                            if (__any_sync(amask, wend - w < (pe - pl) * kRecT)) {
                                const int cnt = (int)((w - lst) / kRecT);
                                rec_store(gl, lst, cnt, SH::list, gpos, over);
                                if (MODE != MODE_LISTS)
                                    rec_eval(sm, lst, cnt, xa, yca, rowa, va, sa, Pa, Ia, Ra2, khf,
                                             Kw, acc);
                                w = lst;
                            }
                            w = rec_scan(sm.e, pl, pe, xd, ya, khf, Kb.four_h2, sgi == 3,
                                         (uint32_t)d, w);
                        }
                    }
                    const int cnt = (int)((w - lst) / kRecT);
                    rec_store(gl, lst, cnt, SH::list, gpos, over);
                    if (MODE != MODE_LISTS)
                        rec_eval(sm, lst, cnt, xa, yca, rowa, va, sa, Pa, Ia, Ra2, khf,
                                 Kw, acc);
                    S.gcnt[t0 + col_i] = over ? (uint8_t)255 : (uint8_t)gpos;
                    if (!over) atomicMax(&sm.lmax, gpos);
                }
            }
        } else if (active && build) {
            S.gcnt[t0 + col_i] = (uint8_t)255;  // no list: this window takes the global path
        }
        if (MODE == MODE_LISTS) continue;  // lists stored: nothing to sum
        if (active && global) {
            // neighbour block too large for shared memory, a chunk with more
            // windows than the table holds, or a list that did not fit: every
            // in-support neighbour from global memory
            const uint32_t ki = __ldg(F.key + i);
            cxa = (int)(ki / (uint32_t)ncy);
            cy = (int)ki - cxa * ncy;
            const float2 la = __ldg(F.loc + i);
            const float2 va = __ldg(F.v + i);
            const float sa = __ldg(F.rho + i);
            Ia = rcp_approx(P.rho0 + sa);
            const float pa = STORED_P ? __ldg(F.p + i) : eos(sa, P);
            acc = Acc4{0.f, 0.f, 0.f, 0.f};
            if constexpr (CASES) {
                // a global-path window may span several columns, and so
                // several cases: the target's own column gives its case
                tcase = __ldg(S.col_case + cxa);
                TileConst Kt = K;
                Kt.c1 = S.cases[tcase].c1;
                Kt.c2 = S.cases[tcase].c2;
                target_global<STORED_P>(F, fstart, wstart, Wl, g, P, Kt, i, cxa, cy, la, va, sa,
                                        pa * Ia, Ia, K.two_rho0 + sa, acc);
            } else {
                target_global<STORED_P>(F, fstart, wstart, Wl, g, P, K, i, cxa, cy, la, va, sa,
                                        pa * Ia, Ia, K.two_rho0 + sa, acc);
            }
        }
        if (active) {
            const float mb = P.m * P.bwen_h;
            const float ax = acc.ax * mb;
            const float ay = fmaf(acc.ay, mb, -(CASES ? S.cases[tcase].g : P.g));
            const float drho = mb * fmaf(-P.k_psi, acc.diff, acc.cont);
            if constexpr (MODE == MODE_FORCES) {
                F.a[i] = make_float2(ax, ay);
                F.drho[i] = drho;
            } else {
                // Integrate_SymplecticCorrector (src/SPH_integration.h:289-309),
                // as in k_pairs_tiled
                const float e = -drho * Ia * dt;
                const float ie = rcp_approx(2.f + e);
                const float s_new = ro_s * ((2.f - e) * ie) - P.rho0 * (2.f * e * ie);
                const float2 nv = make_float2(fmaf(ax, dt, ro_v.x), fmaf(ay, dt, ro_v.y));
                const float hdt = 0.5f * dt;
                const double2 rn = make_double2(ro_r.x + (double)((nv.x + ro_v.x) * hdt),
                                                ro_r.y + (double)((nv.y + ro_v.y) * hdt));
                out.r[i] = rn;
                reinterpret_cast<float2 *>(out.v)[i] = nv;
                reinterpret_cast<float *>(out.rho)[i] = s_new;
                bool resort = false;
                if (out_of_domain_bits(rn, CASES ? S.cases[tcase].box : out.boxb)) {
                    // an erase candidate: its cell kept in case the erase
                    // skips it (the cell of every other particle is found by
                    // the sort, k_hist_kept, which runs only when some
                    // particle needs it; so is its histogram slot)
                    int ncx_, ncy_;
                    uint32_t nk = cell_key(g, rn, (uint32_t)(cxa * ncy + cy), &ncx_, &ncy_);
                    if (!list_removal(out.rm, i)) {
                        nk = (uint32_t)g.ncells;
                        atomicOr(health, kHealthRemoved);
                    }
                    out.key[i] = nk;
                    resort = true;
                }
                if (!(nv.x == nv.x) || !(nv.y == nv.y) || !(s_new == s_new))
                    atomicOr(health, kHealthNan);
                // the new position relative to the kept cell, the pair
                // records of the next pass, and whether the cells must be
                // rebuilt before it
                const float2 ln = make_float2((float)(rn.x - __ldg(g.ax.org + cxa)),
                                              (float)(rn.y - __ldg(g.ay.org + cy)));
                S.nloc[i] = ln;
                const float ib = rcp_approx(P.rho0 + s_new);
                S.nrec.e[i] = make_float4(ln.x, ln.y, (float)cy, ib);
                S.nrec.v[i] = make_float4(nv.x, nv.y, s_new, eos(s_new, P) * ib);
                const float ex = ln.x - lb.x, ey = ln.y - lb.y;
                if (resort || !(fmaf(ex, ex, ey * ey) <= S.sig2)) {
                    *S.need_sort = 1u;
                    if (S.use_cond) cudaGraphSetConditional(S.cond_sort, 1u);
                }
            }
        }
    }
    if (build) {  // the last window's longest list
        __syncthreads();
        if (tid == 0 && nw > 0) table_w[nw - 1].lrows = sm.lmax;
    }
    finish();
}

// the position fields of the fluid records (x, y, row of e) at the binning
// positions (lbin): lists rebuilt from them are the lists that were built
// right after that binning (a restored state whose lists were overwritten
// since)
static __global__ void __launch_bounds__(kBlock)
k_lbin_records(PairRec R, const float2 *__restrict__ lbin, const uint32_t *__restrict__ key,
               const uint32_t *__restrict__ fstart, Grid g) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live(fstart, g.ncells)) return;
    const float2 l = lbin[i];
    const uint32_t k = key[i];
    const int cx = (int)(k / (uint32_t)g.ncy);
    const float row = (float)((int)k - cx * g.ncy);
    float *const e = reinterpret_cast<float *>(R.e + i);
    e[0] = l.x;
    e[1] = l.y;
    e[2] = row;
}

// An uploaded state applied in the current (kept) order: every fluid row's
// position relative to its kept cell and its pair records are formed from
// the uploaded fields, the walls' records from their uploaded densities, and
// `flag` is set when the kept cells cannot stay: a particle more than sigma
// from where it was binned (or not finite), or lists not built after the
// last binning.  The re-binning kernels that follow are gated on `flag`.
static __global__ void __launch_bounds__(kBlock)
k_upload_keep(FluidState<float> F, const uint32_t *__restrict__ fstart, WallState<float> Wl,
              int nw, Grid g, Phys<float> P, const float2 *__restrict__ lbin, float sig2,
              const uint32_t *__restrict__ gen, PairRec RF, PairRec RW,
              uint32_t *__restrict__ flag) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        wall_record(RW, i, Wl.rho[i], P);
        return;
    }
    const int f = i - nw;
    if (f == 0 && __ldg(gen) != __ldg(gen + 1)) *flag = 1u;
    if (f >= n_live(fstart, g.ncells)) return;
    const uint32_t key = F.key[f];
    if (key >= (uint32_t)g.ncells) return;  // a removed row
    const int cx = (int)(key / (uint32_t)g.ncy);
    const int cy = (int)key - cx * g.ncy;
    const float2 ln = cell_local(g, F.r[f], cx, cy);
    F.loc[f] = ln;
    const float2 lb = lbin[f];
    const float ex = ln.x - lb.x, ey = ln.y - lb.y;
    if (!(fmaf(ex, ex, ey * ey) <= sig2)) *flag = 1u;
    const float s = F.rho[f];
    const float2 v = F.v[f];
    const float ib = rcp_approx(P.rho0 + s);
    RF.e[f] = make_float4(ln.x, ln.y, (float)cy, ib);
    RF.v[f] = make_float4(v.x, v.y, s, eos(s, P) * ib);
}

// the sort of a kept-order state (when some particle left its kept cell's
// reach, or the domain): the cell of every particle at its new position (the
// kept cell as the starting guess) and its histogram slot, except the erase
// candidates, whose slots the erase takes; a particle outside the removal box
// that could not be listed keeps the removed key the corrector gave it
template <typename T>
__global__ void __launch_bounds__(kBlock)
k_hist_kept(FluidState<T> X, uint32_t *__restrict__ key, uint32_t *__restrict__ slot,
            uint32_t *__restrict__ counts, const uint8_t *__restrict__ cand,
            const uint32_t *__restrict__ fstart, Grid g, BoxBits box,
            uint32_t *__restrict__ health, const uint32_t *__restrict__ gate,
            uint32_t *__restrict__ runs, const int32_t *__restrict__ col_case,
            const CaseConst *__restrict__ cases) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && runs) atomicAdd(runs, 1u);
    if (i >= n_live(fstart, g.ncells)) return;
    if (cand[X.id[i]]) return;
    const double2 r = X.r[i];
    if (col_case)  // packed cases: the removal box of the particle's case
        box = cases[__ldg(col_case + X.key[i] / (uint32_t)g.ncy)].box;
    uint32_t k;
    if (out_of_domain_bits(r, box)) {
        k = key[i];
    } else {
        int cx, cy;
        k = cell_key(g, r, X.key[i], &cx, &cy);
        if (k == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
        key[i] = k;
    }
    slot[i] = atomicAdd(counts + k, 1u);
}

// the sorted rows (r, v, rho, id, key, loc of S) back into the buffers the
// graph reads (D)
template <typename T>
__global__ void __launch_bounds__(kBlock)
k_copy_rows(FluidState<T> D, const FluidState<T> S, const uint32_t *__restrict__ fstart,
            int ncells, const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int)__ldg(fstart + ncells + 1)) return;
    D.r[i] = S.r[i];
    D.v[i] = S.v[i];
    D.rho[i] = S.rho[i];
    D.id[i] = S.id[i];
    D.key[i] = S.key[i];
    D.loc[i] = S.loc[i];
}

}  // namespace tsph
