// tsph_ale.cu -- the Riemann / ALE-SPH step on the GPU (cases/ALESPH_dambreakLong/
// MUSCL.h path): FP32 fluxes, FP64 integration of omega, omega*rho, omega*v.
//
// State in HBM (fluid, sorted by cell like the WCSPH engine): r FP64, loc
// FP32 (cell-local position), the conserved omega / omega*rho (FP64) and
// omega*v (FP64 x2), their leap-frog copies, the rates (FP32), and the
// derived rho - rho0 and v (FP32) that the flux loop reads.  Walls (one BT
// layer with normals) are static and binned once.
//
// Kernels per step: k_ale_lf1 (leap-frog part one, in place: particles do
// not move), k_ale_grad (one-sided gradients; only for the MUSCL scheme),
// k_ale_flux (the pair loop), k_ale_lf2_bin (part two + out-of-domain +
// cell and histogram slot), then the counting sort (scan, k_place,
// k_ale_rank_scatter).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/tsph.h"
#include "tsph_engine.h"
#include "tsph_grid_host.h"
#include "tsph_kernels.cuh"

namespace tsph {
namespace {

struct AleFluid {
    double2 *r;
    float2 *loc;
    uint32_t *key, *id;
    double *om, *omr;
    double2 *omv;
    double *om_o, *omr_o;
    double2 *omv_o;
    float *dom, *domr;
    float2 *domv;
    float *s;   // rho - rho0
    float2 *v;
    float *ps;  // rho - rho0 at the last Density_to_pressure (the reference's p)
    float *grad;  // 12 per particle, valid until the next re-binning
};

struct AleWalls {
    double2 *r;
    float2 *loc;
    uint32_t *key, *id;
    float2 *n;
    float *s;
};

struct AleConst {
    float h, inv_h, m, c0, rho0, g, dp, four_h2, awen, bwen_h, b_eos;
    float inv_rho0, inv_c0, inv_c02;  // products instead of divisions in the pair terms
    float dx_exact;  // below this |dx| the FP32 cell-local difference may carry the wrong sign
    // |dy| beyond which the rows above / below of a target stop: 2h, plus
    // twice the skin, since on kept cells a cell's y order may be off by two
    // moves of at most the skin each
    float reach;
    float list_r2;  // (2h + 2 skin)^2: the radius of the lists kept between sorts
};

// neighbour lists of the flux kernel kept between sorts (kept cells): per
// target (sorted row i) up to kAleList entries ent[k * nfa + i] (the staged
// index << 2 | row code of its window, which repeats while the cells stay)
// and their count cnt[i] (0xFF: the target takes the global-memory path);
// cta_gen[b] the sort generation CTA b built them for, *gen the current one
// (every sort increments it); lbin the fluid's binning positions, from which
// they are built (2h + 2 skin: complete while every particle is within the
// skin of its binning)
struct AleLists {
    uint16_t *ent;
    uint8_t *cnt;
    uint32_t *cta_gen;
    const uint32_t *gen;
    const float2 *lbin;
    long long nfa;
    int keep;
    uint32_t *gate_clear;  // the fused step's sort word, cleared at the start (or null)
};

// the fused step's part two (and next part one) in the flux kernel's
// epilogue (NEXT): each target's new state goes to D, the spare set (other
// CTAs still read the target's half-step state as a neighbour); the sort
// word of this step is `gate_set` (raised by a move past the skin or a
// removal), `gate_clear_next` the next step's, cleared here (the two
// alternate: a launch cannot clear the word its own blocks raise)
struct AleNext {
    AleFluid D;
    float dtf, hf, rho0, sig2;
    int step;
    BoxBits boxb;
    uint32_t *gate_set, *gate_clear_next, *health;
};

__device__ __forceinline__ float ale_eos(float s, const AleConst &K) {
    const float x = s * K.inv_rho0;
    return K.b_eos * x * (7.f + x * (21.f + x * (35.f + x * (35.f + x * (21.f + x * (7.f + x))))));
}

// W and (dW/dr)/r of the Wendland kernel for 0 < r2 <= 4h^2
__device__ __forceinline__ void ale_wendland(float r2, const AleConst &K, float &W, float &F) {
    const float r = r2 * rsqrtf(r2);
    const float w1 = fmaf(-0.5f * K.inv_h, r, 1.f);
    const float w2 = w1 * w1;
    F = K.bwen_h * w2 * w1;
    W = K.awen * fmaf(2.f * K.inv_h, r, 1.f) * w2 * w2;
}

// MUSCL_superBee slope D, src/_testMUSCL_schemes.h:33-77
__device__ __forceinline__ float superbee(float gFx, float gFy, float gBx, float gBy, float dx,
                                          float dy) {
    const float DF = gFx * dx + gFy * dy, DB = gBx * dx + gBy * dy;
    if (DF > 0.f) return fmaxf(0.f, fmaxf(fminf(2.f * DB, DF), fminf(DB, DF)));
    if (DF < 0.f) return fminf(0.f, fminf(fmaxf(2.f * DB, DF), fmaxf(DB, DF)));
    return 0.f;
}

__device__ __forceinline__ void derive(double om, double omr, double2 omv, float rho0, float &s,
                                       float2 &v) {
    // rho = omega*rho / omega, v = omega*v / (rho omega), src/RALESPH_integration.h:31-32;
    // rho - rho0 from the FP64 numerator keeps its precision in FP32
    const double num = fma(-(double)rho0, om, omr);
    const float omf = (float)om;
    s = (float)num / omf;
    const float omrf = (float)omr;
    v = make_float2((float)omv.x / omrf, (float)omv.y / omrf);
}

__device__ __forceinline__ int n_live_ale(const uint32_t *fstart, int ncells) {
    return (int)__ldg(fstart + ncells);
}

// The leap-frog increments (rate x step, position change v x step) are
// formed in FP32 and added to the FP64 state with one FP64 add: the rates
// and velocities are FP32 values (FP32 pair math, ~1e-6 relative), so the
// FP32 product (6e-8 relative) loses nothing they carry, and GB300 issues
// FP64 at a small fraction of the FP32 rate.  dtf = dt, hf = dt/2 in FP32.
__device__ __forceinline__ double add_f(double x, float rate, float step) {
    return x + (double)(rate * step);
}

// Integrate_LeapFrog_partOne, src/RALESPH_integration.h:10-36 (in place)
__global__ void k_ale_lf1(AleFluid F, const uint32_t *__restrict__ fstart, int ncells, float hf,
                          float rho0) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, ncells)) return;
    const double om = F.om[i], omr = F.omr[i];
    const double2 omv = F.omv[i];
    F.om_o[i] = om;
    F.omr_o[i] = omr;
    F.omv_o[i] = omv;
    const double om2 = add_f(om, F.dom[i], hf), omr2 = add_f(omr, F.domr[i], hf);
    const float2 dv = F.domv[i];
    const double2 omv2 = make_double2(add_f(omv.x, dv.x, hf), add_f(omv.y, dv.y, hf));
    F.om[i] = om2;
    F.omr[i] = omr2;
    F.omv[i] = omv2;
    float s;
    float2 v;
    derive(om2, omr2, omv2, rho0, s, v);
    F.s[i] = s;
    F.v[i] = v;
}

// Integrate_LeapFrog_partTwo, src/RALESPH_integration.h:38-107, for target i:
// returns the new position, the new conserved state goes to D[o].  FORM:
// kLf2Single (the per-function entry point, in place: everything, the
// leap-frog copies and the derived rho, v included); kLf2Moved (the fused
// step before its sort, out of place: no copies, no derived rho, v -- the
// sort derives them from the conserved state; the copies are dead until the
// next part one); kLf2Kept (the fused step on kept cells, in place: derived
// rho, v, no copies, and the rates and the index, which stay, not rewritten);
// kLf2KeptNext (as kLf2Kept, then the next step's part one with the same
// rates and step, src/RALESPH_integration.h:10-36: the new state goes to the
// leap-frog copies, the half-step state and its rho, v to omega, omega*rho,
// omega*v, s, v -- bit for bit what k_ale_lf1 would write next).
enum { kLf2Single = 0, kLf2Moved = 1, kLf2Kept = 2, kLf2KeptNext = 3 };
template <int FORM>
__device__ __forceinline__ double2 lf2(const AleFluid &F, int i, AleFluid D, int o, float dtf,
                                       float hf, int step, float rho0, float &s_out,
                                       float2 &v_out) {
    constexpr bool NEXT = FORM == kLf2KeptNext;
    constexpr bool COPIES = FORM == kLf2Single, DERIVED = FORM != kLf2Moved && !NEXT,
                   MOVE = FORM != kLf2Kept && !NEXT;
    double2 r = F.r[i];
    // the reference's p was computed from the density the fluxes used
    const float s_flux = F.s[i];
    const float2 dv = F.domv[i];
    double om, omr;
    double2 omv;
    // the increments rate x step of part two (as add_f forms them), and the
    // factor that makes them the next part one's rate x dt/2: 1 at step 1
    // (part two's step is dt/2 there), else 1/2 -- dt/2 is dt halved in FP32
    // as in FP64, so (rate x dt) / 2 is rate x dt/2 exactly
    double i0, i1, i2, i3, half_of;
    if (step == 1) {
        const double om0 = F.om[i], omr0 = F.omr[i];
        const double2 omv0 = F.omv[i];
        if (COPIES) {
            D.om_o[o] = om0;
            D.omr_o[o] = omr0;
            D.omv_o[o] = omv0;
        }
        i0 = (double)(F.dom[i] * hf);
        i1 = (double)(F.domr[i] * hf);
        i2 = (double)(dv.x * hf);
        i3 = (double)(dv.y * hf);
        half_of = 1.0;
        om = om0 + i0;
        omr = omr0 + i1;
        omv = make_double2(omv0.x + i2, omv0.y + i3);
        derive(om, omr, omv, rho0, s_out, v_out);
        r = make_double2(add_f(r.x, v_out.x, hf), add_f(r.y, v_out.y, hf));
    } else {
        const float2 v0 = F.v[i];
        r = make_double2(add_f(r.x, v0.x, dtf), add_f(r.y, v0.y, dtf));
        i0 = (double)(F.dom[i] * dtf);
        i1 = (double)(F.domr[i] * dtf);
        i2 = (double)(dv.x * dtf);
        i3 = (double)(dv.y * dtf);
        half_of = 0.5;
        om = F.om_o[i] + i0;
        omr = F.omr_o[i] + i1;
        const double2 o2 = F.omv_o[i];
        omv = make_double2(o2.x + i2, o2.y + i3);
        // NEXT stores the half-step rho, v only (derived below; they carry a
        // NaN of the new state to the caller's check as well)
        if (!NEXT) derive(om, omr, omv, rho0, s_out, v_out);
        if (COPIES) {
            D.om_o[o] = F.om_o[i];
            D.omr_o[o] = F.omr_o[i];
            D.omv_o[o] = o2;
        }
    }
    if (DERIVED) {
        D.s[o] = s_out;
        D.v[o] = v_out;
    }
    if (NEXT) {
        D.om_o[o] = om;
        D.omr_o[o] = omr;
        D.omv_o[o] = omv;
        // the next part one: one rounding of x + increment x factor, as
        // add_f(x, rate, dt/2) rounds x + rate x dt/2
        const double omh = fma(i0, half_of, om), omrh = fma(i1, half_of, omr);
        const double2 omvh = make_double2(fma(i2, half_of, omv.x), fma(i3, half_of, omv.y));
        D.om[o] = omh;
        D.omr[o] = omrh;
        D.omv[o] = omvh;
        float sh;
        float2 vh;
        derive(omh, omrh, omvh, rho0, sh, vh);
        D.s[o] = sh;
        D.v[o] = vh;
        if (step != 1) {
            s_out = sh;
            v_out = vh;
        }
    } else {
        D.om[o] = om;
        D.omr[o] = omr;
        D.omv[o] = omv;
    }
    if (MOVE) {
        D.dom[o] = F.dom[i];
        D.domr[o] = F.domr[i];
        D.domv[o] = dv;
        D.id[o] = F.id[i];
    }
    D.r[o] = r;
    D.ps[o] = s_flux;
    return r;
}

// part two in place (per-function entry point)
__global__ void k_ale_lf2(AleFluid F, const uint32_t *__restrict__ fstart, int ncells, float dtf,
                          float hf, int step, float rho0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, ncells)) return;
    float sn;
    float2 vn;
    lf2<kLf2Single>(F, i, F, i, dtf, hf, step, rho0, sn, vn);
}

// part two out of place + RemoveParticlesOutOfDomain (src/SPH_btdebug.h:4-31)
// + cell and histogram slot of the new position
__global__ void k_ale_lf2_bin(AleFluid F, const uint32_t *__restrict__ fstart, Grid g, float dtf,
                              float hf, int step, float rho0, BoxBits boxb, AleFluid D,
                              uint32_t *__restrict__ key, uint32_t *__restrict__ slot,
                              uint32_t *__restrict__ counts, uint32_t *__restrict__ health) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, g.ncells)) return;
    float sn;
    float2 v;
    const double2 rn = lf2<kLf2Moved>(F, i, D, i, dtf, hf, step, rho0, sn, v);
    if (!(v.x == v.x) || !(v.y == v.y) || !(sn == sn)) atomicOr(health, kHealthNan);
    uint32_t k;
    if (out_of_domain_bits(rn, boxb)) {
        k = (uint32_t)g.ncells;
        atomicOr(health, kHealthRemoved);
    } else {
        int cx, cy;
        k = cell_key(g, rn, F.key[i], &cx, &cy);
        if (k == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
    }
    key[i] = k;
    slot[i] = atomicAdd(counts + k, 1u);
}

// part two in place on kept cells (the fused step between sorts), followed
// by the next step's part one (kLf2KeptNext): the new position's cell-local
// coordinates against the particle's kept cell.  `gate`
// is raised when a particle has moved more than the skin since its binning
// (sig2 = skin^2) or left the domain (RemoveParticlesOutOfDomain,
// src/SPH_btdebug.h:4-31), and the sort that follows runs.
__global__ void k_ale_lf2_keep(AleFluid F, const uint32_t *__restrict__ fstart, Grid g, float dtf,
                               float hf, int step, float rho0, BoxBits boxb,
                               const float2 *__restrict__ lbin, float sig2,
                               uint32_t *__restrict__ gate, uint32_t *__restrict__ health) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, g.ncells)) return;
    float sn;
    float2 v;
    const double2 rn = lf2<kLf2KeptNext>(F, i, F, i, dtf, hf, step, rho0, sn, v);
    if (!(v.x == v.x) || !(v.y == v.y) || !(sn == sn)) atomicOr(health, kHealthNan);
    if (out_of_domain_bits(rn, boxb)) {
        atomicOr(health, kHealthRemoved);
        *gate = 1u;
        return;
    }
    const uint32_t k = F.key[i];
    const int cx = (int)(k / (uint32_t)g.ncy), cy = (int)k - cx * g.ncy;
    const float2 l = cell_local(g, rn, cx, cy);
    F.loc[i] = l;
    const float2 b = lbin[i];
    const float dx = l.x - b.x, dy = l.y - b.y;
    if (!(fmaf(dx, dx, dy * dy) <= sig2)) *gate = 1u;
}

// cell and histogram slot of every live particle for the sort on kept cells
// (runs when `gate` was raised; `runs` counts the sorts); with `remove` (a
// step's sort) out of the domain -> the last bucket.  This and the other gated kernels loop over
// their items grid-stride, so that a small grid skips at little cost.
__global__ void k_ale_hist_gated(AleFluid F, const uint32_t *__restrict__ fstart, Grid g,
                                 BoxBits boxb, int remove, uint32_t *__restrict__ key,
                                 uint32_t *__restrict__ slot, uint32_t *__restrict__ counts,
                                 uint32_t *__restrict__ health, const uint32_t *__restrict__ gate,
                                 unsigned long long *__restrict__ runs) {
    pdl_enter();
    if (gated_off(gate)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(runs, 1ull);
    const int nl = n_live_ale(fstart, g.ncells);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nl; i += gridDim.x * blockDim.x) {
        const double2 r = F.r[i];
        uint32_t k = (uint32_t)g.ncells;
        if (!(remove && out_of_domain_bits(r, boxb))) {
            int cx, cy;
            k = cell_key(g, r, F.key[i], &cx, &cy);
            if (k == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
        }
        key[i] = k;
        slot[i] = atomicAdd(counts + k, 1u);
    }
}

// the sorted state back into the step's arrays after a sort on kept cells
// (the leap-frog copies included: they hold the state at the end of the step)
__global__ void k_ale_copy_gated(AleFluid S, AleFluid D, const uint32_t *__restrict__ fstart,
                                 int ncells, const uint32_t *__restrict__ gate) {
    pdl_enter();
    if (gated_off(gate)) return;
    const int n = (int)fstart[ncells + 1];
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        D.r[j] = S.r[j];
        D.loc[j] = S.loc[j];
        D.key[j] = S.key[j];
        D.id[j] = S.id[j];
        D.om[j] = S.om[j];
        D.omr[j] = S.omr[j];
        D.omv[j] = S.omv[j];
        D.om_o[j] = S.om_o[j];
        D.omr_o[j] = S.omr_o[j];
        D.omv_o[j] = S.omv_o[j];
        D.dom[j] = S.dom[j];
        D.domr[j] = S.domr[j];
        D.domv[j] = S.domv[j];
        D.s[j] = S.s[j];
        D.v[j] = S.v[j];
        D.ps[j] = S.ps[j];
    }
}

// undo a part one applied ahead (k_ale_lf2_keep): the state at the end of
// the step back from the leap-frog copies, rho - rho0 and v derived from it
__global__ void k_ale_unhalf(AleFluid F, const uint32_t *__restrict__ fstart, int ncells,
                             float rho0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, ncells)) return;
    const double om = F.om_o[i], omr = F.omr_o[i];
    const double2 omv = F.omv_o[i];
    F.om[i] = om;
    F.omr[i] = omr;
    F.omv[i] = omv;
    float s;
    float2 v;
    derive(om, omr, omv, rho0, s, v);
    F.s[i] = s;
    F.v[i] = v;
}

// Particle_To_Cell on kept cells: each live particle's cell-local position
// against its kept cell; `gate` raised when one moved more than the skin
// since its binning (sig2 = skin^2) or left its cell's block for good
__global__ void k_ale_relocate(AleFluid F, const uint32_t *__restrict__ fstart, Grid g,
                               const float2 *__restrict__ lbin, float sig2,
                               uint32_t *__restrict__ gate) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, g.ncells)) return;
    const uint32_t k = F.key[i];
    const int cx = (int)(k / (uint32_t)g.ncy), cy = (int)k - cx * g.ncy;
    const float2 l = cell_local(g, F.r[i], cx, cy);
    F.loc[i] = l;
    const float2 b = lbin[i];
    const float dx = l.x - b.x, dy = l.y - b.y;
    if (!(fmaf(dx, dx, dy * dy) <= sig2)) *gate = 1u;
}

// cell key of the current positions (per-function Particle_To_Cell)
__global__ void k_ale_bin(AleFluid F, const uint32_t *__restrict__ fstart, Grid g,
                          uint32_t *__restrict__ key, uint32_t *__restrict__ slot,
                          uint32_t *__restrict__ counts, uint32_t *__restrict__ health) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, g.ncells)) return;
    int cx, cy;
    uint32_t k = F.key[i];
    if (k != (uint32_t)g.ncells) {
        k = cell_key(g, F.r[i], k, &cx, &cy);
        if (k == (uint32_t)g.ncells) atomicOr(health, kHealthEscaped);
    }
    key[i] = k;
    slot[i] = atomicAdd(counts + k, 1u);
}

// rank inside the cell by (y, particle index) and move the record (+ loc,
// and loc as the binning position into lbin).  STEP: after the fused step's
// part two — the leap-frog copies stay behind and rho - rho0, v are derived
// from the conserved state; otherwise (a plain re-binning, or the sort on
// kept cells) every field moves as it is.  `gate` (may be null): runs only
// when it is set.
template <bool STEP>
__global__ void k_ale_rank_scatter(const uint32_t *__restrict__ key, const int *__restrict__ n_ptr,
                                   const uint32_t *__restrict__ start,
                                   const uint32_t *__restrict__ tmp_id,
                                   const uint32_t *__restrict__ tmp_src,
                                   const long long *__restrict__ tmp_y, Grid g, AleFluid S,
                                   AleFluid D, float rho0, float2 *__restrict__ lbin,
                                   const uint32_t *__restrict__ gate, uint32_t *__restrict__ gen) {
    pdl_enter();
    if (gated_off(gate)) return;
    // a new cell order: the flux kernel's kept lists are stale
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(gen, 1u);
    const int n = *n_ptr;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t src = tmp_src[j];
        const uint32_t k = key[src];
        uint32_t f = (uint32_t)j;
        if (k != (uint32_t)g.ncells) {
            const uint32_t lo = start[k], hi = start[k + 1];
            const uint32_t me = tmp_id[j];
            const long long my = tmp_y[j];
            uint32_t rank = 0;
            for (uint32_t m = lo; m < hi; m++) {
                const long long ym = tmp_y[m];
                rank += (ym < my || (ym == my && tmp_id[m] < me)) ? 1u : 0u;
            }
            f = lo + rank;
        }
        const double2 r = S.r[src];
        D.r[f] = r;
        D.key[f] = k;
        D.id[f] = S.id[src];
        if (k < (uint32_t)g.ncells) {
            const int cx = (int)(k / (uint32_t)g.ncy), cy = (int)k - cx * g.ncy;
            const float2 l = cell_local(g, r, cx, cy);
            D.loc[f] = l;
            lbin[f] = l;
        }
        const double om = S.om[src], omr = S.omr[src];
        const double2 omv = S.omv[src];
        D.om[f] = om;
        D.omr[f] = omr;
        D.omv[f] = omv;
        D.dom[f] = S.dom[src];
        D.domr[f] = S.domr[src];
        D.domv[f] = S.domv[src];
        D.ps[f] = S.ps[src];
        if (STEP) {
            float sn;
            float2 vn;
            derive(om, omr, omv, rho0, sn, vn);
            D.s[f] = sn;
            D.v[f] = vn;
        } else {
            D.om_o[f] = S.om_o[src];
            D.omr_o[f] = S.omr_o[src];
            D.omv_o[f] = S.omv_o[src];
            D.s[f] = S.s[src];
            D.v[f] = S.v[src];
        }
    }
}

// neighbour at larger x (dx = x_a - x_b < 0) -> forward sums, smaller x ->
// backward sums, equal x -> neither (src/_testMUSCL_gradientApprox.h:135-178).
// The split is discontinuous in x_a - x_b, so its sign is taken from the FP64
// positions whenever the FP32 difference is within its rounding error
// (particles of one lattice column stay within ~1e-8 m of each other for
// many steps).
__device__ __forceinline__ float exact_side(float dx, double xa, const double2 *rb, int j,
                                            const AleConst &K) {
    if (fabsf(dx) >= K.dx_exact) return dx;
    const double d = xa - __ldg(&rb[j].x);
    return d < 0.0 ? -1.f : (d > 0.0 ? 1.f : 0.f);
}

__device__ __forceinline__ void accumulate_side(float gF[6], float gB[6], float dx,
                                                const float t[6]) {
    const float wf = dx < 0.f ? 1.f : 0.f, wb = dx > 0.f ? 1.f : 0.f;
#pragma unroll
    for (int q = 0; q < 6; q++) {
        gF[q] = fmaf(wf, t[q], gF[q]);
        gB[q] = fmaf(wb, t[q], gB[q]);
    }
}

// Kernel_gradient_approx, src/_testMUSCL_gradientApprox.h:10-231: forward
// (neighbour at larger x) / backward one-sided gradients of rho, vx, vy,
// walls through their normals, x2; zero when no neighbour is in support.
__global__ void __launch_bounds__(kBlock)
k_ale_grad(AleFluid F, const uint32_t *__restrict__ fstart, const uint32_t *__restrict__ wstart,
           AleWalls Wl, Grid g, AleConst K) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, g.ncells)) return;
    const uint32_t key = F.key[i];
    const int cx = (int)(key / (uint32_t)g.ncy), cy = (int)key - cx * g.ncy;
    const float2 la = F.loc[i], va = F.v[i];
    const float sa = F.s[i];
    const double xa = F.r[i].x;
    float gF[6] = {0, 0, 0, 0, 0, 0}, gB[6] = {0, 0, 0, 0, 0, 0};
    float gamma = 0.f;
    for (int dxi = 0; dxi < 3; dxi++) {
        const int col = cx + dxi - 1;
        if (col < 0 || col >= g.ncx) continue;
        for (int dyi = 0; dyi < 3; dyi++) {
            const int row = cy + dyi - 1;
            if (row < 0 || row >= g.ncy) continue;
            const int c = col * g.ncy + row;
            const float bx = la.x + (float)(1 - dxi) * g.khf, by = la.y + (float)(1 - dyi) * g.khf;
            for (int j = (int)__ldg(wstart + c); j < (int)__ldg(wstart + c + 1); j++) {
                const float2 lb = __ldg(Wl.loc + j);
                const float dx = bx - lb.x, dy = by - lb.y;
                const float r2 = fmaf(dx, dx, dy * dy);
                if (!(r2 <= K.four_h2)) continue;
                float W, Fk;
                if (r2 == 0.f) { W = K.awen; Fk = 0.f; } else ale_wendland(r2, K, W, Fk);
                const float2 n = __ldg(Wl.n + j);
                const float nbx = -n.x, nby = -n.y;
                const float sb = __ldg(Wl.s + j);
                const float wdp = W * K.dp;
                const float t[6] = {(sb - sa) * nbx * wdp, (sb - sa) * nby * wdp,
                                    -va.x * nbx * wdp,     -va.x * nby * wdp,
                                    -va.y * nbx * wdp,     -va.y * nby * wdp};
                accumulate_side(gF, gB, exact_side(dx, xa, Wl.r, j, K), t);
                gamma += W * K.m / (K.rho0 + sb);
            }
            for (int j = (int)__ldg(fstart + c); j < (int)__ldg(fstart + c + 1); j++) {
                if (j == i) continue;
                const float2 lb = __ldg(F.loc + j);
                const float dx = bx - lb.x, dy = by - lb.y;
                const float r2 = fmaf(dx, dx, dy * dy);
                if (!(r2 <= K.four_h2)) continue;
                float W, Fk;
                if (r2 == 0.f) { W = K.awen; Fk = 0.f; } else ale_wendland(r2, K, W, Fk);
                const float sb = __ldg(F.s + j);
                const float2 vb = __ldg(F.v + j);
                const float nom = (float)__ldg(F.om + j);
                const float dWx = dx * Fk, dWy = dy * Fk;
                const float ds = (sb - sa) * nom, dvx = (vb.x - va.x) * nom,
                            dvy = (vb.y - va.y) * nom;
                const float t[6] = {ds * dWx, ds * dWy, dvx * dWx, dvx * dWy, dvy * dWx, dvy * dWy};
                accumulate_side(gF, gB, exact_side(dx, xa, F.r, j, K), t);
                gamma += W * K.m / (K.rho0 + sb);
            }
        }
    }
    float *o = F.grad + (size_t)12 * i;
    for (int q = 0; q < 6; q++) {
        o[q] = gamma == 0.f ? 0.f : gF[q] * 2.f;
        o[6 + q] = gamma == 0.f ? 0.f : gB[q] * 2.f;
    }
}

// does fluid particle j (sorted index) have any neighbour with W > 0?
__device__ bool ale_has_support(const AleFluid &F, const uint32_t *fstart, const uint32_t *wstart,
                                const AleWalls &Wl, const Grid &g, const AleConst &K, int j) {
    const uint32_t key = F.key[j];
    const int cx = (int)(key / (uint32_t)g.ncy), cy = (int)key - cx * g.ncy;
    const float2 la = F.loc[j];
    for (int dxi = 0; dxi < 3; dxi++) {
        const int col = cx + dxi - 1;
        if (col < 0 || col >= g.ncx) continue;
        for (int dyi = 0; dyi < 3; dyi++) {
            const int row = cy + dyi - 1;
            if (row < 0 || row >= g.ncy) continue;
            const int c = col * g.ncy + row;
            const float bx = la.x + (float)(1 - dxi) * g.khf, by = la.y + (float)(1 - dyi) * g.khf;
            for (int kind = 0; kind < 2; kind++) {
                const uint32_t *st = kind ? fstart : wstart;
                for (int n = (int)st[c]; n < (int)st[c + 1]; n++) {
                    if (kind && n == j) continue;
                    const float2 lb = kind ? F.loc[n] : Wl.loc[n];
                    const float dx = bx - lb.x, dy = by - lb.y;
                    if (fmaf(dx, dx, dy * dy) < K.four_h2) return true;
                }
            }
        }
    }
    return false;
}

// Compute_Forces(particles, dt), src/_testMUSCL_interaction.h:13-324, FP32.
// SCHEME 0 (as written): the interface states are the particle states and the
// neighbour's velocity is the active particle's (:184-200 with MUSCL_final
// returning its third argument), so vL = vR = v_a . n_ab.  SCHEME 1: the
// superbee MUSCL states of both particles (left of a, right of b).
template <int SCHEME>
__global__ void __launch_bounds__(kBlock)
k_ale_flux(AleFluid F, const uint32_t *__restrict__ fstart, const uint32_t *__restrict__ wstart,
           AleWalls Wl, Grid g, AleConst K) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_live_ale(fstart, g.ncells)) return;
    const uint32_t key = F.key[i];
    const int cx = (int)(key / (uint32_t)g.ncy), cy = (int)key - cx * g.ncy;
    const float2 la = F.loc[i], va = F.v[i];
    const float sa = F.s[i];
    const float rhoa = K.rho0 + sa;
    const float ao = (float)F.om[i];
    float gA[12];
    if (SCHEME == 1)
        for (int q = 0; q < 12; q++) gA[q] = F.grad[(size_t)12 * i + q];
    float dom = 0.f, domr = 0.f, dvx_s = 0.f, dvy_s = 0.f, gamma = 0.f;
    for (int dxi = 0; dxi < 3; dxi++) {
        const int col = cx + dxi - 1;
        if (col < 0 || col >= g.ncx) continue;
        for (int dyi = 0; dyi < 3; dyi++) {
            const int row = cy + dyi - 1;
            if (row < 0 || row >= g.ncy) continue;
            const int c = col * g.ncy + row;
            const float bx = la.x + (float)(1 - dxi) * g.khf, by = la.y + (float)(1 - dyi) * g.khf;
            // BT wall neighbours, :253-265, :275-281
            for (int j = (int)__ldg(wstart + c); j < (int)__ldg(wstart + c + 1); j++) {
                const float2 lb = __ldg(Wl.loc + j);
                const float dx = bx - lb.x, dy = by - lb.y;
                const float r2 = fmaf(dx, dx, dy * dy);
                if (!(r2 <= K.four_h2) || r2 == 0.f) continue;
                float W, Fk;
                ale_wendland(r2, K, W, Fk);
                const float2 n = __ldg(Wl.n + j);
                const float nbx = -n.x, nby = -n.y;
                const float vn = va.x * nbx + va.y * nby;
                const float ps = ale_eos(sa + rhoa * vn / K.c0, K);
                const float wdp = W * K.dp;
                dvx_s -= 2.f * wdp * (ps * nbx);
                dvy_s -= 2.f * wdp * (ps * nby);
                dom -= vn * wdp;
                gamma += W * K.m / (K.rho0 + __ldg(Wl.s + j));
            }
            for (int j = (int)__ldg(fstart + c); j < (int)__ldg(fstart + c + 1); j++) {
                if (j == i) continue;
                const float2 lb = __ldg(F.loc + j);
                const float dx = bx - lb.x, dy = by - lb.y;
                const float r2 = fmaf(dx, dx, dy * dy);
                if (!(r2 <= K.four_h2) || r2 == 0.f) continue;
                float W, Fk;
                ale_wendland(r2, K, W, Fk);
                const float sb = __ldg(F.s + j);
                const float2 vb = __ldg(F.v + j);
                const float no = (float)__ldg(F.om + j);
                const float dWx = dx * Fk, dWy = dy * Fk;
                const float inv_r = rsqrtf(r2);
                const float nx = -dx * inv_r, ny = -dy * inv_r;  // pair normal
                float vL, vR, sL, sR;
                if (SCHEME == 0) {
                    vL = va.x * nx + va.y * ny;
                    vR = vL;
                    sL = sa;
                    sR = sb;
                } else {
                    float gB[12];
                    for (int q = 0; q < 12; q++) gB[q] = __ldg(F.grad + (size_t)12 * j + q);
                    sL = sa - superbee(gA[0], gA[1], gA[6], gA[7], dx, dy);
                    const float vLx = va.x - superbee(gA[2], gA[3], gA[8], gA[9], dx, dy);
                    const float vLy = va.y - superbee(gA[4], gA[5], gA[10], gA[11], dx, dy);
                    sR = sb + superbee(gB[0], gB[1], gB[6], gB[7], dx, dy);
                    const float vRx = vb.x + superbee(gB[2], gB[3], gB[8], gB[9], dx, dy);
                    const float vRy = vb.y + superbee(gB[4], gB[5], gB[10], gB[11], dx, dy);
                    vL = vLx * nx + vLy * ny;
                    vR = vRx * nx + vRy * ny;
                }
                const float rbar = K.rho0 + 0.5f * (sa + sb);
                // velRiemannLinearized / densRiemannLinearized,
                // src/ALESPH_riemann_solver.h:6-18,86-96
                const float vss = 0.5f * (vR + vL) - 0.5f * (sR - sL) * K.c0 / rbar;
                const float ss = 0.5f * (sL + sR) + 0.5f * (vL - vR) * rbar / K.c0;
                const float ps = ale_eos(ss, K);
                const float rhos = K.rho0 + ss;
                const float h2 = 0.5f * (vL + vR);
                const float vsx = nx * vss + (0.5f * (va.x + vb.x) - nx * h2);
                const float vsy = ny * vss + (0.5f * (va.y + vb.y) - ny * h2);
                const float ex = vsx - va.x, ey = vsy - va.y;
                const float vsdW = ex * dWx + ey * dWy;
                dvx_s -= 2.f * no * ((rhos * vsx * ex + ps) * dWx + (rhos * vsx * ey) * dWy);
                dvy_s -= 2.f * no * ((rhos * vsy * ex) * dWx + (rhos * vsy * ey + ps) * dWy);
                const float dvdW = (va.x - vb.x) * dWx + (va.y - vb.y) * dWy;
                dom -= dvdW * no;
                domr -= 2.f * rhos * no * vsdW;
                gamma += W * K.m / (K.rho0 + sb);
            }
        }
    }
    bool zero = gamma == 0.f;
    if (zero) {
        // the reference's gamma_sum is not reset between the particles of a
        // cell (:49, :299): a particle without neighbours still gets the
        // gravity term when an earlier particle of its cell had some
        const uint32_t me = F.id[i];
        const int c = cx * g.ncy + cy;
        for (int j = (int)fstart[c]; j < (int)fstart[c + 1] && zero; j++)
            if (j != i && F.id[j] < me && ale_has_support(F, fstart, wstart, Wl, g, K, j)) zero = false;
    }
    if (zero) {
        F.dom[i] = 0.f;
        F.domr[i] = 0.f;
        F.domv[i] = make_float2(0.f, 0.f);
    } else {
        F.dom[i] = dom * ao;
        F.domr[i] = domr * ao;
        F.domv[i] = make_float2(dvx_s * ao, dvy_s * ao - K.g * ao * rhoa);
    }
}


// ---- the as-written flux loop as a shared-memory tiled gather (the layout
// of the WCSPH pair kernel): a CTA takes 128 consecutive sorted fluid
// particles, stages the 3 x (rows + 2) neighbour cells, builds each target's
// in-support list, then evaluates the pairs.  Cells are sorted by y, so the
// rows above and below stop once |dy| > 2h.
constexpr int kAleT = 128;
constexpr int kAleRows = 16;
constexpr int kAleCap = 608;
constexpr int kAleList = 36;

struct AleTile {
    float2 loc[kAleCap];
    float4 q[kAleCap];  // fluid {vx, vy, rho - rho0, omega}; wall {-nx, -ny, rho - rho0, -1}
    int foff[3][kAleRows + 3];
    int woff[3][kAleRows + 3];
    float offy[4];  // y offset of a neighbour row: below, own, above (list code 0, 1, 2)
    uint16_t list[kAleList * kAleT];
};

__device__ __forceinline__ float ale_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

struct AleAcc {
    float dom, domr, dvx, dvy;
    bool any;  // some neighbour with W > 0 (gamma_sum != 0)
};

// one pair term.  SCHEME 0 (as written, src/_testMUSCL_interaction.h:184-296
// with MUSCL_final's states): rho_L = rho_a, rho_R = rho_b, v_L = v_R =
// v_a . n.  SCHEME 2 (first order, src/RALESPH_interaction.h:132-256): v_R =
// v_b . n, rho* with densRiemannLinearizedWithLimiter
// (src/ALESPH_riemann_solver.h:20-34), walls with the linear equation of
// state Compute_Pressure2 (src/SPH_pressure.h:24-34).
template <int SCHEME>
__device__ __forceinline__ void ale_pair(float dx, float dy, float2 va, float sa, float rhoa,
                                         float4 qb, const AleConst &K, AleAcc &acc) {
    const float r2 = fmaf(dx, dx, dy * dy);
    // a kept list holds neighbours up to 2h + 2 skin and the target itself
    if (!(r2 > 0.f && r2 <= K.four_h2)) return;
    const float inv_r = rsqrtf(r2);
    const float r = r2 * inv_r;
    const float w1 = fmaf(-0.5f * K.inv_h, r, 1.f);
    const float w2 = w1 * w1;
    const float W = K.awen * fmaf(2.f * K.inv_h, r, 1.f) * w2 * w2;
    acc.any |= W > 0.f;
    if (qb.w < 0.f) {
        // BT wall: rho* = rho_a (1 + v_a . n_b / c0), pressure along n_b
        const float vn = va.x * qb.x + va.y * qb.y;
        const float sw = fmaf(rhoa * vn, K.inv_c0, sa);
        const float ps = SCHEME == 2 ? K.c0 * K.c0 * sw : ale_eos(sw, K);
        const float wdp = W * K.dp;
        acc.dvx = fmaf(-2.f * wdp * ps, qb.x, acc.dvx);
        acc.dvy = fmaf(-2.f * wdp * ps, qb.y, acc.dvy);
        acc.dom = fmaf(-vn, wdp, acc.dom);
        return;
    }
    const float F = K.bwen_h * w2 * w1;
    const float dWx = dx * F, dWy = dy * F;
    const float sb = qb.z;
    const float ob = qb.w;
    const float nx = -dx * inv_r, ny = -dy * inv_r;
    float vsx, vsy, ss;
    if (SCHEME == 2) {
        const float vL = va.x * nx + va.y * ny, vR = qb.x * nx + qb.y * ny;
        const float rbar = K.rho0 + 0.5f * (sa + sb);
        const float vss = 0.5f * (vR + vL) - 0.5f * (sb - sa) * K.c0 * ale_rcp(rbar);
        const float d = vL - vR;
        const float beta = fminf(3.f * fmaxf(d, 0.f), K.c0);
        ss = 0.5f * (sa + sb) + 0.5f * beta * d * rbar * K.inv_c02;
        const float t = vss - 0.5f * (vL + vR);
        vsx = fmaf(nx, t, 0.5f * (va.x + qb.x));
        vsy = fmaf(ny, t, 0.5f * (va.y + qb.y));
    } else {
        // v* = v_L n - (rho_R - rho_L) c0 / (2 rho_bar) n + mean tangential
        // part; rho* = mean density (v_L = v_R)
        const float k = -0.5f * (sb - sa) * K.c0 * ale_rcp(K.rho0 + 0.5f * (sa + sb));
        ss = 0.5f * (sa + sb);
        vsx = fmaf(nx, k, 0.5f * (va.x + qb.x));
        vsy = fmaf(ny, k, 0.5f * (va.y + qb.y));
    }
    const float ps = ale_eos(ss, K);
    const float rhos = K.rho0 + ss;
    const float ex = vsx - va.x, ey = vsy - va.y;
    const float t2 = 2.f * ob;
    acc.dvx = fmaf(-t2, fmaf(fmaf(rhos * vsx, ex, ps), dWx, rhos * vsx * ey * dWy), acc.dvx);
    acc.dvy = fmaf(-t2, fmaf(rhos * vsy * ex, dWx, fmaf(rhos * vsy, ey, ps) * dWy), acc.dvy);
    acc.dom = fmaf(-ob, (va.x - qb.x) * dWx + (va.y - qb.y) * dWy, acc.dom);
    acc.domr = fmaf(-t2 * rhos, ex * dWx + ey * dWy, acc.domr);
}

// the bounded append of a row range that could overflow the list: one
// candidate at a time, at most up to the list's end (0 < r^2 <= h2: the
// particle itself and coincident particles excluded; with `with_zero`
// r^2 <= h2, for the lists kept between sorts); a candidate past the end
// sets `overflow`.  Inlined: out of line, its calls from the unrolled loops
// made the kernel spill registers.
static __device__ __forceinline__ uint16_t *append_bounded_ale(const float2 *loc, uint16_t *lst,
                                                            uint16_t *w, int j0, int j1,
                                                            uint32_t code, float bx, float by,
                                                            float h2, bool with_zero,
                                                            bool &overflow) {
    uint16_t *const wend = lst + kAleList * kAleT;
    for (int j = j0; j < j1; j++) {
        const float2 lb = loc[j];
        const float dx = bx - lb.x, dy = by - lb.y;
        const float r2 = fmaf(dx, dx, dy * dy);
        if (with_zero ? r2 <= h2 : in_support(r2, __float_as_uint(h2))) {
            if (w < wend) {
                *w = (uint16_t)(((uint32_t)j << 2) | code);
                w += kAleT;
            } else {
                overflow = true;
            }
        }
    }
    return w;
}

__device__ __forceinline__ void l2_prefetch(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// slot e of a window's staged block (segments walls 0, fluid 0, walls 1,
// ...): the row j it stages, whether a wall, and x of its cell's origin
// relative to the centre column's
__device__ __forceinline__ void ale_slot(int e, const int *w0, const int *f0, const int *wb,
                                         const int *fb, float khf, int &j, bool &wall,
                                         float &xs) {
    j = e + w0[0];
    wall = true;
    xs = -khf;
    if (e >= fb[0]) { j = e - fb[0] + f0[0]; wall = false; }
    if (e >= wb[1]) { j = e - wb[1] + w0[1]; wall = true; xs = 0.f; }
    if (e >= fb[1]) { j = e - fb[1] + f0[1]; wall = false; }
    if (e >= wb[2]) { j = e - wb[2] + w0[2]; wall = true; xs = khf; }
    if (e >= fb[2]) { j = e - fb[2] + f0[2]; wall = false; }
}

template <int SCHEME, bool NEXT>
__global__ void __launch_bounds__(kAleT, 8)
k_ale_flux_tiled(AleFluid F, const uint32_t *__restrict__ fstart,
                 const uint32_t *__restrict__ wstart, AleWalls Wl, Grid g, AleConst K,
                 AleLists L, AleNext N) {
    __shared__ AleTile sm;
    pdl_enter();
    const int tid = threadIdx.x;
    // the step's sort word, raised again by its part two (this launch runs
    // after the last sort's kernels have read it); fused: the next step's
    if (blockIdx.x == 0 && tid == 0) {
        if (NEXT) *N.gate_clear_next = 0u;
        else if (L.gate_clear) *L.gate_clear = 0u;
    }
    const int ncy = g.ncy;
    const int nl = n_live_ale(fstart, g.ncells);
    const int t0 = blockIdx.x * kAleT;
    if (t0 >= nl) return;
    const int t1 = min(t0 + kAleT, nl);
    // lists: mode 0 built per window (kept cells off), 1 built from the
    // binning positions and stored (first call after a sort), 2 the stored
    // ones (the cells, hence the windows, unchanged since)
    int mode = 0;
    if (L.keep) mode = L.cta_gen[blockIdx.x] == *L.gen ? 2 : 1;
    if (tid < 4) sm.offy[tid] = tid < 3 ? (float)(1 - tid) * g.khf : 0.f;
    const float khf = g.khf;
    const float reach = K.reach;
    // the CTA's last target: when it lies in the first window's column and
    // rows, that window is the whole CTA (no further lookups for its end)
    const uint32_t klast = __ldg(F.key + t1 - 1);
    const int cxl = (int)(klast / (uint32_t)ncy);
    const int cyll = (int)klast - cxl * ncy;
    int cur = t0;
    int rows = kAleRows;
    while (cur < t1) {
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
        const uint32_t ki = active ? __ldg(F.key + i) : 0u;  // fetched with the offsets
        if (NEXT && active) {
            // the target's state for the part two in the epilogue, on its way
            // to L2 while the pair sums run (no registers held)
            l2_prefetch(F.r + i);
            l2_prefetch(F.om_o + i);
            l2_prefetch(F.omr_o + i);
            l2_prefetch(F.omv_o + i);
            l2_prefetch(F.v + i);
            l2_prefetch(F.s + i);
            l2_prefetch(L.lbin + i);
        }
        __syncthreads();
        for (int e = tid; e < 3 * (nr + 1); e += kAleT) {
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
        if (tot > kAleCap && rows > 1) {
            rows = (rows + 1) >> 1;
            continue;
        }
        AleAcc acc = {0.f, 0.f, 0.f, 0.f, false};
        bool done = false;
        float2 va = make_float2(0.f, 0.f);
        float sa = 0.f;
        if (tot <= kAleCap) {
            // slot e of the block: segments walls 0, fluid 0, walls 1, ...;
            // all of a thread's loads go out before its first store; x is
            // staged relative to the centre column, y to the particle's cell
            constexpr int kStage = (kAleCap + kAleT - 1) / kAleT;
            float2 st_l[kStage], st_v[kStage];
            float st_s[kStage];
            double st_o[kStage];
            bool st_w[kStage];
            const float2 *const floc = mode == 1 ? L.lbin : F.loc;
#pragma unroll
            for (int u = 0; u < kStage; u++) {
                const int e = tid + u * kAleT;
                int j;
                bool wall;
                float xs;
                ale_slot(e, w0, f0, wb, fb, khf, j, wall, xs);
                st_w[u] = wall;
                st_l[u] = make_float2(0.f, 0.f);
                st_v[u] = make_float2(0.f, 0.f);
                st_s[u] = 0.f;
                st_o[u] = 0.0;
                if (e < tot) {
                    st_l[u] = __ldg((wall ? Wl.loc : floc) + j);
                    st_l[u].x += xs;
                    st_v[u] = __ldg((wall ? Wl.n : F.v) + j);
                    st_s[u] = __ldg((wall ? Wl.s : F.s) + j);
                    if (!wall) st_o[u] = __ldg(F.om + j);
                }
            }
#pragma unroll
            for (int u = 0; u < kStage; u++) {
                const int e = tid + u * kAleT;
                if (e < tot) {
                    sm.loc[e] = st_l[u];
                    // walls: {-n, s, -1}; fluid: {v, s, omega}
                    sm.q[e] = st_w[u] ? make_float4(-st_v[u].x, -st_v[u].y, st_s[u], -1.f)
                                      : make_float4(st_v[u].x, st_v[u].y, st_s[u], (float)st_o[u]);
                }
            }
            __syncthreads();
            bool overflow = false;
            int cnt = 0;
            uint16_t *const lst = sm.list + tid;
            if (active && mode == 2) {
                // the list stored after the last sort
                const int c = (int)L.cnt[i];
                if (c > kAleList) {
                    overflow = true;
                } else {
                    for (int k = 0; k < c; k++) lst[k * kAleT] = L.ent[(size_t)k * L.nfa + i];
                    cnt = c;
                }
            } else if (active) {
                const int cy = (int)ki - cx * ncy;
                const int own = fb[1] + (i - f0[1]);
                const float2 la = sm.loc[own];
                // neighbours into the list (entry: staged index << 2 | row
                // code): mode 0 the in-support ones (0 < r^2 <= 4h^2), mode 1
                // those within 2h + 2 skin of the binning positions (the
                // target itself included: the pair terms skip r = 0); per
                // column the rows below, own and above are staged ranges
                // [R0, R1), [R1, R2), [R2, R3).  A range that could overflow
                // the list is appended one at a time, bounded (a target with
                // more than kAleList neighbours takes the global-memory path)
                const float h2 = mode == 1 ? K.list_r2 : K.four_h2;
                uint16_t *const wend = lst + kAleList * kAleT;
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
                        if (wend - w < (R2 - R1) * kAleT)
                            w = append_bounded_ale(sm.loc, lst, w, R1, R2, 1u, la.x, la.y, h2,
                                                   mode == 1, overflow);
                        else if (d == 1 && kind == 1 && mode == 0)
                            w = scan_own<kAleT, true>(sm.loc, R1, R2, la.x, la.y, h2, w);
                        else
                            w = scan_own<kAleT, false>(sm.loc, R1, R2, la.x, la.y, h2, w);
                        if (wend - w < (R3 - R2) * kAleT)
                            w = append_bounded_ale(sm.loc, lst, w, R2, R3, 2u, la.x, by_a, h2,
                                                   mode == 1, overflow);
                        else
                            w = scan_above<kAleT>(sm.loc, R2, R3, la.x, by_a, h2, reach, w);
                        if (wend - w < (R1 - R0) * kAleT)
                            w = append_bounded_ale(sm.loc, lst, w, R0, R1, 0u, la.x, by_b, h2,
                                                   mode == 1, overflow);
                        else
                            w = scan_below<kAleT>(sm.loc, R0, R1, la.x, by_b, h2, reach, w);
                    }
                }
                cnt = (int)((w - lst) / kAleT);
                if (mode == 1) {
                    L.cnt[i] = overflow ? (uint8_t)0xFF : (uint8_t)cnt;
                    if (!overflow)
                        for (int k = 0; k < cnt; k++) L.ent[(size_t)k * L.nfa + i] = lst[k * kAleT];
                }
            }
            if (mode == 1) {
                // the pair terms at the current positions: the fluid's staged
                // positions again (the walls' do not move)
                __syncthreads();
                for (int e = tid; e < tot; e += kAleT) {
                    int j;
                    bool wall;
                    float xs;
                    ale_slot(e, w0, f0, wb, fb, khf, j, wall, xs);
                    if (!wall) {
                        float2 l = __ldg(F.loc + j);
                        l.x += xs;
                        sm.loc[e] = l;
                    }
                }
                __syncthreads();
            }
            if (active && !overflow) {
                const int own = fb[1] + (i - f0[1]);
                const float2 la = sm.loc[own];
                const float4 qa = sm.q[own];
                va = make_float2(qa.x, qa.y);
                sa = qa.z;
                const float rhoa = K.rho0 + sa;
                for (int k = 0; k < cnt; k++) {
                    const uint32_t e = lst[k * kAleT];
                    const int j = (int)(e >> 2);
                    const float oy = sm.offy[e & 3u];
                    const float2 lb = sm.loc[j];
                    ale_pair<SCHEME>(la.x - lb.x, (la.y + oy) - lb.y, va, sa, rhoa, sm.q[j], K,
                                     acc);
                }
                done = true;
            }
        }
        if (active && !done) {
            // window too dense for shared memory, or list overflow: from global memory
            const int cy = (int)ki - cx * ncy;
            const float2 la = __ldg(F.loc + i);
            va = __ldg(F.v + i);
            sa = __ldg(F.s + i);
            const float rhoa = K.rho0 + sa;
            acc = {0.f, 0.f, 0.f, 0.f, false};
            for (int dxi = 0; dxi < 3; dxi++) {
                const int col = cx + dxi - 1;
                if (col < 0 || col >= g.ncx) continue;
                for (int dyi = 0; dyi < 3; dyi++) {
                    const int row = cy + dyi - 1;
                    if (row < 0 || row >= ncy) continue;
                    const int c = col * ncy + row;
                    const float bx = la.x + (float)(1 - dxi) * g.khf,
                                by = la.y + (float)(1 - dyi) * g.khf;
                    for (int j = (int)__ldg(wstart + c); j < (int)__ldg(wstart + c + 1); j++) {
                        const float2 lb = __ldg(Wl.loc + j);
                        const float dx = bx - lb.x, dy = by - lb.y;
                        const float r2 = fmaf(dx, dx, dy * dy);
                        if (!(r2 <= K.four_h2) || r2 == 0.f) continue;
                        const float2 n = __ldg(Wl.n + j);
                        ale_pair<SCHEME>(dx, dy, va, sa, rhoa, make_float4(-n.x, -n.y, __ldg(Wl.s + j), -1.f),
                                 K, acc);
                    }
                    for (int j = (int)__ldg(fstart + c); j < (int)__ldg(fstart + c + 1); j++) {
                        if (j == i) continue;
                        const float2 lb = __ldg(F.loc + j);
                        const float dx = bx - lb.x, dy = by - lb.y;
                        const float r2 = fmaf(dx, dx, dy * dy);
                        if (!(r2 <= K.four_h2) || r2 == 0.f) continue;
                        const float2 vb = __ldg(F.v + j);
                        ale_pair<SCHEME>(dx, dy, va, sa, rhoa,
                                 make_float4(vb.x, vb.y, __ldg(F.s + j), (float)__ldg(F.om + j)), K,
                                 acc);
                    }
                }
            }
        }
        if (active) {
            const int cy = (int)ki - cx * ncy;
            bool zero = !acc.any;
            if (zero) {
                // gamma_sum is not reset between the particles of a cell
                // (src/_testMUSCL_interaction.h:49, :299)
                const uint32_t me = F.id[i];
                const int c = cx * ncy + cy;
                for (int j = (int)fstart[c]; j < (int)fstart[c + 1] && zero; j++)
                    if (j != i && F.id[j] < me && ale_has_support(F, fstart, wstart, Wl, g, K, j))
                        zero = false;
            }
            float rd = 0.f, rr = 0.f;
            float2 rv = make_float2(0.f, 0.f);
            if (!zero) {
                const float ao = (float)F.om[i];
                rd = acc.dom * ao;
                rr = acc.domr * ao;
                rv = make_float2(acc.dvx * ao, acc.dvy * ao - K.g * ao * (K.rho0 + sa));
            }
            F.dom[i] = rd;
            F.domr[i] = rr;
            F.domv[i] = rv;
            if (NEXT) {
                // k_ale_lf2_keep for this target, into the spare set
                float sn;
                float2 vn;
                const double2 rn = lf2<kLf2KeptNext>(F, i, N.D, i, N.dtf, N.hf, N.step, N.rho0, sn, vn);
                N.D.dom[i] = rd;
                N.D.domr[i] = rr;
                N.D.domv[i] = rv;
                N.D.key[i] = ki;
                N.D.id[i] = F.id[i];
                if (!(vn.x == vn.x) || !(vn.y == vn.y) || !(sn == sn)) atomicOr(N.health, kHealthNan);
                if (out_of_domain_bits(rn, N.boxb)) {
                    atomicOr(N.health, kHealthRemoved);
                    *N.gate_set = 1u;
                } else {
                    const float2 l = cell_local(g, rn, cx, cy);
                    N.D.loc[i] = l;
                    const float2 b = L.lbin[i];
                    const float ex = l.x - b.x, ey = l.y - b.y;
                    if (!(fmaf(ex, ex, ey * ey) <= N.sig2)) *N.gate_set = 1u;
                }
            }
        }
        cur = we;
        rows = kAleRows;
    }
    // (the generation changes only with a sort, never during this launch)
    if (mode == 1 && tid == 0) L.cta_gen[blockIdx.x] = *L.gen;
}

#define ACK(call)                                                                 \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
            return TSPH_ERR_CUDA;                                                 \
        }                                                                         \
    } while (0)

inline int nblk(long long n, int b = kBlock) { return (int)std::max<long long>(1, (n + b - 1) / b); }

}  // namespace

// host-side ALE system: particles, grid tables, device buffers
// ---------------------------------------------------------- host staging
// Download / upload through staging arrays indexed by particle (the
// reference's order): the device writes (reads) each field at its particle's
// index, so the host copies whole arrays, with no host-side sort.
struct AleStage {
    double *r = nullptr, *v = nullptr, *rho = nullptr, *p = nullptr, *om = nullptr,
           *omr = nullptr, *omv = nullptr, *dom = nullptr, *domr = nullptr, *domv = nullptr,
           *grad = nullptr;
    int32_t *type = nullptr;
    uint8_t *alive = nullptr;
};

// every live particle (walls, then live fluid rows) writes the requested
// fields at its index and marks itself alive; values as the reference holds
// them (walls: v = 0, omega = dp^2, omega rho = rho dp^2, rates and gradients
// 0; p the equation of state of the density the last fluxes used)
__global__ void k_ale_export(AleFluid F, const uint32_t *__restrict__ fstart, int ncells,
                             AleWalls Wl, int nw, AleStage S, double rho0, double dp2,
                             double b_eos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool wall = i < nw;
    const int j = wall ? i : i - nw;
    if (!wall && j >= n_live_ale(fstart, ncells)) return;
    const uint32_t id = wall ? Wl.id[j] : F.id[j];
    const double rh = rho0 + (double)(wall ? Wl.s[j] : F.s[j]);
    if (S.r) {
        const double2 x = wall ? Wl.r[j] : F.r[j];
        S.r[2 * id] = x.x;
        S.r[2 * id + 1] = x.y;
    }
    if (S.v) {
        const float2 u = wall ? make_float2(0.f, 0.f) : F.v[j];
        S.v[2 * id] = (double)u.x;
        S.v[2 * id + 1] = (double)u.y;
    }
    if (S.rho) S.rho[id] = rh;
    if (S.p) {
        const double x = (wall ? rh : rho0 + (double)F.ps[j]) / rho0;
        S.p[id] = b_eos * (pow(x, 7.) - 1);
    }
    if (S.om) S.om[id] = wall ? dp2 : F.om[j];
    if (S.omr) S.omr[id] = wall ? rh * dp2 : F.omr[j];
    if (S.omv) {
        const double2 q = wall ? make_double2(0., 0.) : F.omv[j];
        S.omv[2 * id] = q.x;
        S.omv[2 * id + 1] = q.y;
    }
    if (S.dom) S.dom[id] = wall ? 0. : (double)F.dom[j];
    if (S.domr) S.domr[id] = wall ? 0. : (double)F.domr[j];
    if (S.domv) {
        const float2 q = wall ? make_float2(0.f, 0.f) : F.domv[j];
        S.domv[2 * id] = (double)q.x;
        S.domv[2 * id + 1] = (double)q.y;
    }
    if (S.grad)
        for (int q = 0; q < 12; q++) S.grad[12 * (size_t)id + q] = wall ? 0. : (double)F.grad[12 * (size_t)j + q];
    if (S.type) S.type[id] = wall ? 1 : 0;
    S.alive[id] = 1;
}

// new volume, density, velocity, position of every live fluid row from the
// staged host arrays (the reference's order), with the conserved quantities
// following: omega first (same rho = omega rho / omega, same v = omega v /
// (rho omega)), then rho, v, r
__global__ void k_ale_import(AleFluid F, const uint32_t *__restrict__ fstart, int ncells,
                             AleStage S, double rho0, int nw, int ntot,
                             uint32_t *__restrict__ health) {
    // a staged upload (health given) applies only while every index is live,
    // else TSPH_HEALTH_UPLOAD and nothing changes
    if (health && (int)fstart[ncells] + nw != ntot) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(health, kHealthUpload);
        return;
    }
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_live_ale(fstart, ncells)) return;
    const uint32_t i = F.id[j];
    double om = F.om[j], omr = F.omr[j];
    double2 omv = F.omv[j];
    if (S.om) {
        const double f = S.om[i] / om;
        om = S.om[i];
        omr *= f;
        omv = make_double2(omv.x * f, omv.y * f);
    }
    if (S.rho) {
        omr = S.rho[i] * om;
        const float sv = (float)(S.rho[i] - rho0);
        F.s[j] = sv;
        F.ps[j] = sv;
    }
    if (S.v) {
        omv = make_double2(S.v[2 * i] * om, S.v[2 * i + 1] * om);
        F.v[j] = make_float2((float)S.v[2 * i], (float)S.v[2 * i + 1]);
    }
    if (S.r) F.r[j] = make_double2(S.r[2 * i], S.r[2 * i + 1]);
    F.om[j] = om;
    F.omr[j] = omr;
    F.omv[j] = omv;
}

class AleEngine {
  public:
    // host setup
    double h = 0, kap = 0, cs = 0, rho0 = 0, visco = 0, delta = 0, dp = 0, m = 0;
    double x0 = 0, xm = 0, y0 = 0, ym = 0, kh = 0, of = 0;
    int ncx = 0, ncy = 0, ncells = 0;
    std::vector<long long> bx, by;
    std::vector<double> ox, oy;
    std::vector<int> type;
    std::vector<double> r, v, rho, p, nrm;
    int scheme = TSPH_ALE_AS_WRITTEN;
    bool divided = false, built = false, cells = false;
    cudaStream_t st = nullptr;
    bool own = false;

    // device
    int nf = 0, nw = 0, ntot = 0;
    std::vector<void *> allocs;
    AleFluid A{}, B{};  // current sorted state, spare
    AleWalls W{};
    Grid grid{};
    AleConst K{};
    uint32_t *fstart = nullptr, *wstart = nullptr, *counts = nullptr, *tiles = nullptr;
    uint32_t *keyB = nullptr, *slotB = nullptr, *tmp_id = nullptr, *tmp_src = nullptr;
    long long *tmp_y = nullptr;
    uint32_t *health = nullptr;
    // kept cells (the fused step): the cells of the last binning stay while
    // every particle is within `skin` of where it was binned (lbin: its
    // cell-local position then) and none left the domain; `gate` raised by
    // part two runs the sort, `sort_runs` counts those sorts
    bool keep = true;
    float skin = 0.f;
    float2 *lbin = nullptr;
    uint32_t *gate = nullptr;
    uint32_t *gate2 = nullptr;  // the fused steps' two alternating sort words
    int gate_parity = 0;
    unsigned long long *sort_runs = nullptr;
    int gated_blocks = 4 * 152;  // grid of a gated launch: 4 blocks per SM
    // the flux kernel's lists kept between sorts (AleLists)
    uint16_t *list_ent = nullptr;
    uint8_t *list_cnt = nullptr;
    uint32_t *list_cta_gen = nullptr, *list_gen = nullptr;
    long long list_nfa = 0;
    // the leap-frog copies (omega_o, ...) hold part one's values: false after
    // a fused step (its re-binning leaves them behind)
    bool copies_valid = true;
    // a fused step on kept cells ends with the next step's part one applied
    // (for a step of half_dt): omega, omega*rho, omega*v, s, v hold the
    // half-step state and the leap-frog copies the state at the end of the
    // step; normalize() puts the end-of-step state back
    bool half = false;
    double half_dt = 0.0;
    // pipelined transfers (r, v, rho): the download's and the upload's own
    // staging sets, copy streams and events; `binned`: a sort has given every
    // live particle its cell (kept-cell re-binning needs one)
    AleStage dstg{}, ustg{};
    cudaStream_t cs_d = nullptr, cs_u = nullptr;
    cudaEvent_t ev_x = nullptr, ev_d = nullptr, ev_up = nullptr, ev_imp = nullptr;
    bool d_pending = false, up_pending = false, binned = false;
    int up_mask = 0;
    float *grad = nullptr;
    AleStage stg{};  // download / upload staging (allocated on first use)
    long long *dbx = nullptr, *dby = nullptr;
    double *dox = nullptr, *doy = nullptr;

    ~AleEngine() {
        release();
        for (cudaStream_t q : {cs_d, cs_u})
            if (q) cudaStreamDestroy(q);
        for (cudaEvent_t q : {ev_x, ev_d, ev_up, ev_imp})
            if (q) cudaEventDestroy(q);
        if (own && st) cudaStreamDestroy(st);
    }

    void release() {
        // copies still in flight read or write the staging sets: done first
        if (d_pending) cudaEventSynchronize(ev_d);
        if (cs_u) cudaStreamSynchronize(cs_u);
        if (st) cudaStreamSynchronize(st);
        for (void *q : allocs) cudaFree(q);
        allocs.clear();
        stg = AleStage{};
        dstg = AleStage{};
        ustg = AleStage{};
        built = false;
        half = false;
        d_pending = false;
        up_pending = false;
        binned = false;
    }

    // a launch with programmatic dependent launch: the kernel (which starts
    // with pdl_enter) is scheduled while the previous one finishes
    template <typename... KA, typename... Args>
    int alaunch(void (*kern)(KA...), int grid, int block, std::string &err, Args... args) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3((unsigned)block);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        ACK(cudaLaunchKernelEx(&cfg, kern, args...));
        return 0;
    }

    // the state at the end of the last step (undo a part one applied ahead)
    int normalize(std::string &err) {
        if (!half) return 0;
        k_ale_unhalf<<<nblk(nf), kBlock, 0, st>>>(A, fstart, ncells, (float)rho0);
        ACK(cudaGetLastError());
        half = false;
        return 0;
    }

    template <typename P> int alloc(P **q, size_t n, std::string &err) {
        void *x = nullptr;
        cudaError_t e = cudaMalloc(&x, std::max<size_t>(n, 1) * sizeof(P));
        if (e != cudaSuccess) {
            err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
            return TSPH_ERR_NOMEM;
        }
        allocs.push_back(x);
        *q = static_cast<P *>(x);
        return 0;
    }

    int alloc_fluid(AleFluid &X, std::string &err) {
        int rc;
        if ((rc = alloc(&X.r, nf, err)) || (rc = alloc(&X.loc, nf, err)) ||
            (rc = alloc(&X.key, nf, err)) || (rc = alloc(&X.id, nf, err)) ||
            (rc = alloc(&X.om, nf, err)) || (rc = alloc(&X.omr, nf, err)) ||
            (rc = alloc(&X.omv, nf, err)) || (rc = alloc(&X.om_o, nf, err)) ||
            (rc = alloc(&X.omr_o, nf, err)) || (rc = alloc(&X.omv_o, nf, err)) ||
            (rc = alloc(&X.dom, nf, err)) || (rc = alloc(&X.domr, nf, err)) ||
            (rc = alloc(&X.domv, nf, err)) || (rc = alloc(&X.s, nf, err)) ||
            (rc = alloc(&X.v, nf, err)) || (rc = alloc(&X.ps, nf, err)))
            return rc;
        X.grad = grad;
        return 0;
    }

    int build(std::string &err) {
        release();
        const int n = (int)type.size();
        ntot = n;
        std::vector<int> fl, wl;
        for (int i = 0; i < n; i++) (type[i] == 1 ? wl : fl).push_back(i);
        nf = (int)fl.size();
        nw = (int)wl.size();
        if ((ncells + 1 + kScanTile - 1) / kScanTile > kScanTile) {
            err = "grid too large for the scan";
            return TSPH_ERR_UNSUPPORTED;
        }
        K.h = (float)h;
        K.inv_h = (float)(1.0 / h);
        K.m = (float)m;
        K.c0 = (float)cs;
        K.rho0 = (float)rho0;
        K.g = 9.81f;
        K.dp = (float)dp;
        K.four_h2 = (float)(4.0 * h * h);
        K.awen = (float)(0.557 / (h * h));
        K.bwen_h = (float)((double)(float)(-2.7852 / (h * h * h)) / h);
        K.b_eos = (float)(cs * cs * rho0 / 7.0);
        {
            int dev = 0, sms = 0;
            ACK(cudaGetDevice(&dev));
            ACK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            if (sms > 0) gated_blocks = 4 * sms;
        }
        K.inv_rho0 = (float)(1.0 / rho0);
        K.inv_c0 = (float)(1.0 / cs);
        K.inv_c02 = (float)(1.0 / (cs * cs));
        // FP32 x_a - x_b from cell-local positions: a few ulps of kh
        K.dx_exact = (float)(4e-6 * kh);
        // the move allowed between two binnings: every pair within 2h stays
        // inside the 3 x 3 cell block (kh >= 2h + 2 skin) with a margin
        skin = (float)std::max(0.0, 0.95 * 0.5 * (kh - 2.0 * h));
        K.reach = 2.f * K.h * 1.0001f + 2.f * skin;
        {
            const double rl = 2.0 * h + 2.0 * (double)skin;
            K.list_r2 = (float)(rl * rl);
        }
        int rc;
        if ((rc = alloc(&grad, (size_t)12 * nf, err))) return rc;
        ACK(cudaMemset(grad, 0, sizeof(float) * 12 * std::max(nf, 1)));
        if ((rc = alloc_fluid(A, err)) || (rc = alloc_fluid(B, err))) return rc;
        if ((rc = alloc(&fstart, ncells + 2, err)) || (rc = alloc(&wstart, ncells + 1, err)) ||
            (rc = alloc(&counts, ncells + 1, err)) ||
            (rc = alloc(&tiles, (ncells + 1 + kScanTile - 1) / kScanTile, err)) ||
            (rc = alloc(&keyB, nf, err)) || (rc = alloc(&slotB, nf, err)) ||
            (rc = alloc(&tmp_id, nf, err)) || (rc = alloc(&tmp_src, nf, err)) ||
            (rc = alloc(&tmp_y, nf, err)) ||
            (rc = alloc(&health, 1, err)) || (rc = alloc(&lbin, nf, err)) ||
            (rc = alloc(&gate, 1, err)) || (rc = alloc(&gate2, 2, err)) ||
            (rc = alloc(&sort_runs, 1, err)) ||
            (rc = alloc(&list_ent, (size_t)kAleList * (size_t)(nblk(nf, kAleT) * kAleT), err)) ||
            (rc = alloc(&list_cnt, nf, err)) ||
            (rc = alloc(&list_cta_gen, nblk(nf, kAleT), err)) || (rc = alloc(&list_gen, 1, err)) ||
            (rc = alloc(&dbx, bx.size(), err)) ||
            (rc = alloc(&dby, by.size(), err)) || (rc = alloc(&dox, ox.size(), err)) ||
            (rc = alloc(&doy, oy.size(), err)))
            return rc;
        ACK(cudaMemcpy(dbx, bx.data(), 8 * bx.size(), cudaMemcpyHostToDevice));
        ACK(cudaMemcpy(dby, by.data(), 8 * by.size(), cudaMemcpyHostToDevice));
        ACK(cudaMemcpy(dox, ox.data(), 8 * ox.size(), cudaMemcpyHostToDevice));
        ACK(cudaMemcpy(doy, oy.data(), 8 * oy.size(), cudaMemcpyHostToDevice));
        ACK(cudaMemset(counts, 0, 4 * (size_t)(ncells + 1)));
        ACK(cudaMemset(health, 0, 4));
        ACK(cudaMemset(gate, 0, 4));
        ACK(cudaMemset(gate2, 0, 8));
        gate_parity = 0;
        ACK(cudaMemset(sort_runs, 0, 8));
        list_nfa = (long long)nblk(nf, kAleT) * kAleT;
        ACK(cudaMemset(list_cta_gen, 0xFF, 4 * (size_t)nblk(nf, kAleT)));
        ACK(cudaMemset(list_gen, 0, 4));
        grid.ax = Axis{dbx, dox, ncx};
        grid.ay = Axis{dby, doy, ncy};
        grid.ncx = ncx;
        grid.ncy = ncy;
        grid.ncells = ncells;
        grid.khf = (float)kh;
        // fluid in index order (ALESPH_Add_particle values)
        {
            std::vector<double2> R(nf), OMV(nf);
            std::vector<double> OM(nf), OMR(nf);
            std::vector<float> S(nf), Z(nf, 0.f);
            std::vector<float2> V(nf), Z2(nf, make_float2(0.f, 0.f));
            std::vector<uint32_t> ID(nf), KEY(nf, 0u);
            const double dp2 = dp * dp;
            for (int k = 0; k < nf; k++) {
                const int i = fl[k];
                R[k] = make_double2(r[2 * i], r[2 * i + 1]);
                OM[k] = dp2;
                OMV[k] = make_double2(v[2 * i] * dp2, v[2 * i + 1] * dp2);
                OMR[k] = rho[i] * dp2;
                S[k] = (float)(rho[i] - rho0);
                V[k] = make_float2((float)v[2 * i], (float)v[2 * i + 1]);
                ID[k] = (uint32_t)i;
            }
            if (nf) {
                ACK(cudaMemcpy(A.r, R.data(), 16 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.om, OM.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.om_o, OM.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.omr, OMR.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.omr_o, OMR.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.omv, OMV.data(), 16 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.omv_o, OMV.data(), 16 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.s, S.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.ps, S.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.v, V.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.dom, Z.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.domr, Z.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.domv, Z2.data(), 8 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.id, ID.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(A.key, KEY.data(), 4 * (size_t)nf, cudaMemcpyHostToDevice));
            }
            std::vector<uint32_t> fs(ncells + 2, 0u);
            fs[ncells] = (uint32_t)nf;
            fs[ncells + 1] = (uint32_t)nf;
            ACK(cudaMemcpy(fstart, fs.data(), 4 * fs.size(), cudaMemcpyHostToDevice));
        }
        // walls, binned once on the host (by cell, then index)
        {
            auto cell_of = [](double x, const std::vector<long long> &b) -> int {
                const long long o = ordered_bits(x);
                if (o < b.front()) return -1;
                if (o >= b.back()) return (int)b.size() - 1;
                return (int)(std::upper_bound(b.begin(), b.end(), o) - b.begin()) - 1;
            };
            std::vector<std::pair<uint32_t, int>> ord;
            for (int i : wl) {
                const int cx = cell_of(r[2 * i], bx), cy = cell_of(r[2 * i + 1], by);
                if (cx < 0 || cy < 0 || cx >= ncx || cy >= ncy) {
                    err = "wall particle " + std::to_string(i) + " lies outside the cell grid";
                    return TSPH_ERR_ARG;
                }
                ord.push_back({(uint32_t)(cy + cx * ncy), i});
            }
            std::sort(ord.begin(), ord.end());
            if ((rc = alloc(&W.r, nw, err)) || (rc = alloc(&W.loc, nw, err)) ||
                (rc = alloc(&W.key, nw, err)) || (rc = alloc(&W.id, nw, err)) ||
                (rc = alloc(&W.n, nw, err)) || (rc = alloc(&W.s, nw, err)))
                return rc;
            std::vector<double2> R(nw);
            std::vector<float2> L(nw), N(nw);
            std::vector<uint32_t> KEY(nw), ID(nw), ws(ncells + 1, 0u);
            std::vector<float> S(nw);
            for (int k = 0; k < nw; k++) {
                const int i = ord[k].second;
                const uint32_t c = ord[k].first;
                const int cx = (int)(c / ncy), cy = (int)(c % ncy);
                R[k] = make_double2(r[2 * i], r[2 * i + 1]);
                L[k] = make_float2((float)(r[2 * i] - ox[cx]), (float)(r[2 * i + 1] - oy[cy]));
                KEY[k] = c;
                ID[k] = (uint32_t)i;
                N[k] = make_float2((float)nrm[2 * i], (float)nrm[2 * i + 1]);
                S[k] = (float)(rho[i] - rho0);
                ws[c + 1]++;
            }
            for (int c = 0; c < ncells; c++) ws[c + 1] += ws[c];
            if (nw) {
                ACK(cudaMemcpy(W.r, R.data(), 16 * (size_t)nw, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(W.loc, L.data(), 8 * (size_t)nw, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(W.key, KEY.data(), 4 * (size_t)nw, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(W.id, ID.data(), 4 * (size_t)nw, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(W.n, N.data(), 8 * (size_t)nw, cudaMemcpyHostToDevice));
                ACK(cudaMemcpy(W.s, S.data(), 4 * (size_t)nw, cudaMemcpyHostToDevice));
            }
            ACK(cudaMemcpy(wstart, ws.data(), 4 * ws.size(), cudaMemcpyHostToDevice));
        }
        ACK(cudaDeviceSynchronize());
        built = true;
        cells = false;
        return 0;
    }

    // counting sort of X (keys in keyB/slotB, histogram in counts) into Y;
    // with `g` every kernel runs only when the word it points to is set
    int sort(AleFluid X, AleFluid Y, bool step_sort, std::string &err,
             const uint32_t *g = nullptr) {
        const int n = ncells + 1;
        const int nt = (n + kScanTile - 1) / kScanTile;
        // gated: grid-stride kernels on a small grid (cheap to skip)
        const int bn = g ? std::min(nblk(n), gated_blocks) : nblk(n);
        const int bf = g ? std::min(nblk(nf), gated_blocks) : nblk(nf);
        int rc;
        const int *ntot_ = reinterpret_cast<const int *>(fstart + ncells + 1);
        const long long *ty = tmp_y;
        if ((rc = alaunch(k_scan_tiles_clear, nt, kScanThreads, err, counts, fstart, tiles, n, g)) ||
            (rc = alaunch(k_scan_add_tiles, bn, kBlock, err, fstart, (const uint32_t *)tiles, nt,
                          n, g)) ||
            (rc = alaunch(k_place, bf, kBlock, err, (const uint32_t *)keyB,
                          (const uint32_t *)slotB, (const uint32_t *)X.id, ntot_,
                          (const uint32_t *)fstart, tmp_id, tmp_src, (const double2 *)X.r, tmp_y,
                          g)))
            return rc;
        if (step_sort)
            rc = alaunch(k_ale_rank_scatter<true>, bf, kBlock, err, (const uint32_t *)keyB, ntot_,
                         (const uint32_t *)fstart, (const uint32_t *)tmp_id,
                         (const uint32_t *)tmp_src, ty, grid, X, Y, (float)rho0, lbin, g,
                         list_gen);
        else
            rc = alaunch(k_ale_rank_scatter<false>, bf, kBlock, err, (const uint32_t *)keyB, ntot_,
                         (const uint32_t *)fstart, (const uint32_t *)tmp_id,
                         (const uint32_t *)tmp_src, ty, grid, X, Y, (float)rho0, lbin, g,
                         list_gen);
        return rc;
    }

    int particle_to_cell(std::string &err) {
        if (int rc = normalize(err)) return rc;
        if (up_pending) {
            // the staged upload first (every index live, checked on the device)
            AleStage S{};
            if (up_mask & TSPH_ALE_F_R) S.r = ustg.r;
            if (up_mask & TSPH_ALE_F_V) S.v = ustg.v;
            if (up_mask & TSPH_ALE_F_RHO) S.rho = ustg.rho;
            ACK(cudaStreamWaitEvent(st, ev_up, 0));
            k_ale_import<<<nblk(nf), kBlock, 0, st>>>(A, fstart, ncells, S, rho0, nw, ntot, health);
            ACK(cudaGetLastError());
            ACK(cudaEventRecord(ev_imp, st));
            up_pending = false;
        }
        if (keep && skin > 0.f && binned) {
            // kept cells: the sort only when a particle moved past the skin
            const Box box{x0, xm, y0, ym};
            const int bg = std::min(nblk(nf), gated_blocks);
            ACK(cudaMemsetAsync(gate, 0, 4, st));
            k_ale_relocate<<<nblk(nf), kBlock, 0, st>>>(A, fstart, grid, lbin, skin * skin, gate);
            k_ale_hist_gated<<<bg, kBlock, 0, st>>>(A, fstart, grid, make_box_bits(box), 0, keyB,
                                                    slotB, counts, health, gate, sort_runs);
            if (int rc = sort(A, B, false, err, gate)) return rc;
            k_ale_copy_gated<<<bg, kBlock, 0, st>>>(B, A, fstart, ncells, gate);
            ACK(cudaGetLastError());
            cells = true;
            return 0;
        }
        k_ale_bin<<<nblk(nf), kBlock, 0, st>>>(A, fstart, grid, keyB, slotB, counts, health);
        int rc = sort(A, B, false, err);
        if (rc) return rc;
        std::swap(A, B);
        cells = true;
        binned = true;
        return 0;
    }

    int gradient(std::string &err) {
        if (int rc = no_staged_upload(err)) return rc;
        if (int rc = normalize(err)) return rc;
        k_ale_grad<<<nblk(nf), kBlock, 0, st>>>(A, fstart, wstart, W, grid, K);
        ACK(cudaGetLastError());
        return 0;
    }

    // the flux kernel's kept lists: on with kept cells (the cells, hence
    // its windows, change only with a sort, which makes them stale)
    AleLists lists(uint32_t *clear = nullptr) const {
        return AleLists{list_ent, list_cnt, list_cta_gen, list_gen, lbin, list_nfa,
                        keep && skin > 0.f ? 1 : 0, clear};
    }
    uint32_t *gate_clear = nullptr;  // set by the fused step around its forces()

    int forces(std::string &err) {
        if (int rc = no_staged_upload(err)) return rc;
        if (int rc = normalize(err)) return rc;
        if (scheme == TSPH_ALE_MUSCL)
            k_ale_flux<1><<<nblk(nf), kBlock, 0, st>>>(A, fstart, wstart, W, grid, K);
        else
            return alaunch(scheme == TSPH_ALE_FIRST_ORDER ? k_ale_flux_tiled<2, false>
                                                          : k_ale_flux_tiled<0, false>,
                           nblk(nf, kAleT), kAleT, err, A, (const uint32_t *)fstart,
                           (const uint32_t *)wstart, W, grid, K, lists(gate_clear), AleNext{});
        ACK(cudaGetLastError());
        return 0;
    }

    int lf1(double dt, std::string &err) {
        if (int rc = no_staged_upload(err)) return rc;
        if (half && half_dt == dt) {
            // applied ahead by the last fused step, bit for bit
            half = false;
            copies_valid = true;
            return 0;
        }
        if (int rc = normalize(err)) return rc;
        if (int rc = alaunch(k_ale_lf1, nblk(nf), kBlock, err, A, (const uint32_t *)fstart, ncells,
                             (float)(dt * 0.5), (float)rho0))
            return rc;
        copies_valid = true;
        return 0;
    }

    int lf2(double dt, int step, std::string &err) {
        if (int rc = no_staged_upload(err)) return rc;
        if (int rc = normalize(err)) return rc;
        if (step != 1 && !copies_valid) {
            err = "Integrate_LeapFrog_partTwo (step > 1) needs part one of the same step first";
            return TSPH_ERR_STATE;
        }
        k_ale_lf2<<<nblk(nf), kBlock, 0, st>>>(A, fstart, ncells, (float)dt, (float)(dt * 0.5),
                                               step, (float)rho0);
        ACK(cudaGetLastError());
        cells = false;
        return 0;
    }

    // the RUN body nsteps times.  On kept cells (`keep`, the default) part two
    // runs in place and the sort only when a particle moved more than the
    // skin or left the domain; otherwise every step re-bins and sorts (the
    // reference's cell order every step)
    int step(double dt, int step0, int nsteps, std::string &err) {
        if (int rc = no_staged_upload(err)) return rc;
        const Box box{x0, xm, y0, ym};
        const BoxBits boxb = make_box_bits(box);
        const bool kept = keep && skin > 0.f;
        for (int k = 1; k <= nsteps; k++) {
            const int stp = step0 + k;
            int rc;
            // part one: applied ahead by the last step, or now
            if (half && (stp == 1 || half_dt != dt) && (rc = normalize(err))) return rc;
            if (stp > 1 && !half && (rc = lf1(dt, err))) return rc;
            half = false;
            if (scheme == TSPH_ALE_MUSCL && (rc = gradient(err))) return rc;
            if (kept && scheme != TSPH_ALE_MUSCL) {
                // fluxes and part two (+ the next part one) in one launch,
                // the new state into the spare set, which becomes the state
                uint32_t *gs = gate2 + gate_parity, *gn = gate2 + (gate_parity ^ 1);
                AleNext nx{};
                nx.D = B;
                nx.dtf = (float)dt;
                nx.hf = (float)(dt * 0.5);
                nx.rho0 = (float)rho0;
                nx.sig2 = skin * skin;
                nx.step = stp;
                nx.boxb = boxb;
                nx.gate_set = gs;
                nx.gate_clear_next = gn;
                nx.health = health;
                const int bg = std::min(nblk(nf), gated_blocks);
                if ((rc = alaunch(scheme == TSPH_ALE_FIRST_ORDER ? k_ale_flux_tiled<2, true>
                                                                 : k_ale_flux_tiled<0, true>,
                                  nblk(nf, kAleT), kAleT, err, A, (const uint32_t *)fstart,
                                  (const uint32_t *)wstart, W, grid, K, lists(), nx)))
                    return rc;
                std::swap(A, B);
                if ((rc = alaunch(k_ale_hist_gated, bg, kBlock, err, A, (const uint32_t *)fstart,
                                  grid, boxb, 1, keyB, slotB, counts, health,
                                  (const uint32_t *)gs, sort_runs)) ||
                    (rc = sort(A, B, false, err, gs)) ||
                    (rc = alaunch(k_ale_copy_gated, bg, kBlock, err, B, A, (const uint32_t *)fstart,
                                  ncells, (const uint32_t *)gs)))
                    return rc;
                gate_parity ^= 1;
                half = true;
                half_dt = dt;
                continue;
            }
            // on kept cells the tiled flux kernel clears the sort word
            const bool tiled = scheme != TSPH_ALE_MUSCL;
            gate_clear = kept && tiled ? gate : nullptr;
            rc = forces(err);
            gate_clear = nullptr;
            if (rc) return rc;
            if (kept) {
                if (!tiled) ACK(cudaMemsetAsync(gate, 0, 4, st));
                const int bg = std::min(nblk(nf), gated_blocks);
                if ((rc = alaunch(k_ale_lf2_keep, nblk(nf), kBlock, err, A, (const uint32_t *)fstart,
                                  grid, (float)dt, (float)(dt * 0.5), stp, (float)rho0, boxb,
                                  (const float2 *)lbin, skin * skin, gate, health)) ||
                    (rc = alaunch(k_ale_hist_gated, bg, kBlock, err, A, (const uint32_t *)fstart,
                                  grid, boxb, 1, keyB, slotB, counts, health,
                                  (const uint32_t *)gate, sort_runs)) ||
                    (rc = sort(A, B, false, err, gate)) ||
                    (rc = alaunch(k_ale_copy_gated, bg, kBlock, err, B, A, (const uint32_t *)fstart,
                                  ncells, (const uint32_t *)gate)))
                    return rc;
                half = true;
                half_dt = dt;
            } else {
                k_ale_lf2_bin<<<nblk(nf), kBlock, 0, st>>>(A, fstart, grid, (float)dt,
                                                           (float)(dt * 0.5), stp, (float)rho0,
                                                           boxb, B, keyB, slotB, counts, health);
                if ((rc = sort(B, A, true, err))) return rc;
            }
        }
        ACK(cudaGetLastError());
        cells = true;
        if (nsteps > 0) copies_valid = false;
        return 0;
    }

    int np_live(int *np, std::string &err) {
        uint32_t nl = 0;
        ACK(cudaMemcpyAsync(&nl, fstart + ncells, 4, cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        *np = (int)nl + nw;
        return 0;
    }

    template <typename P> int stage(P **q, size_t per, std::string &err) {
        return *q ? 0 : alloc(q, per * (size_t)ntot, err);
    }

    // state in the reference's order: the device writes every requested field
    // at its particle's index (k_ale_export); with every particle live the
    // host copies whole arrays, otherwise it keeps the live ones
    int download(int mask, const tsph_ale_host_state *o, std::string &err) {
        int rc;
        if ((rc = no_staged_upload(err)) || (rc = normalize(err))) return rc;
        AleStage S{};
        struct Want {
            int bit;
            double *host;
            double **dev;
            int width;
        };
        const Want want[] = {{TSPH_ALE_F_R, o->r, &stg.r, 2},
                             {TSPH_ALE_F_V, o->v, &stg.v, 2},
                             {TSPH_ALE_F_RHO, o->rho, &stg.rho, 1},
                             {TSPH_ALE_F_P, o->p, &stg.p, 1},
                             {TSPH_ALE_F_OMEGA, o->omega, &stg.om, 1},
                             {TSPH_ALE_F_OMEGARHO, o->omegarho, &stg.omr, 1},
                             {TSPH_ALE_F_OMEGAV, o->omegav, &stg.omv, 2},
                             {TSPH_ALE_F_RATES, o->domega, &stg.dom, 1},
                             {TSPH_ALE_F_RATES, o->domegarho, &stg.domr, 1},
                             {TSPH_ALE_F_RATES, o->domegav, &stg.domv, 2},
                             {TSPH_ALE_F_GRAD, o->grad, &stg.grad, 12}};
        double **sp[] = {&S.r, &S.v, &S.rho, &S.p, &S.om, &S.omr, &S.omv, &S.dom, &S.domr,
                         &S.domv, &S.grad};
        for (int k = 0; k < 11; k++) {
            if (!(mask & want[k].bit) || !want[k].host) continue;
            if ((rc = stage(want[k].dev, (size_t)want[k].width, err))) return rc;
            *sp[k] = *want[k].dev;
        }
        const bool want_type = (mask & TSPH_ALE_F_TYPE) && o->type;
        if (want_type) {
            if ((rc = stage(&stg.type, 1, err))) return rc;
            S.type = stg.type;
        }
        if ((rc = stage(&stg.alive, 1, err))) return rc;
        S.alive = stg.alive;
        ACK(cudaMemsetAsync(stg.alive, 0, (size_t)ntot, st));
        k_ale_export<<<nblk(nw + nf), kBlock, 0, st>>>(A, fstart, ncells, W, nw, S, rho0, dp * dp,
                                                       cs * cs * rho0 / 7.);
        ACK(cudaGetLastError());
        uint32_t nl = 0;
        ACK(cudaMemcpyAsync(&nl, fstart + ncells, 4, cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        const bool dense = (long long)nl + nw == (long long)ntot;
        std::vector<uint8_t> alive;
        if (!dense) {
            alive.resize(ntot);
            ACK(cudaMemcpyAsync(alive.data(), stg.alive, (size_t)ntot, cudaMemcpyDeviceToHost, st));
            ACK(cudaStreamSynchronize(st));
        }
        std::vector<double> tmp;
        for (int k = 0; k < 11; k++) {
            if (!*sp[k]) continue;
            const size_t wdt = (size_t)want[k].width;
            if (dense) {
                ACK(cudaMemcpyAsync(want[k].host, *sp[k], 8 * wdt * ntot, cudaMemcpyDeviceToHost, st));
                continue;
            }
            tmp.resize(wdt * ntot);
            ACK(cudaMemcpyAsync(tmp.data(), *sp[k], 8 * wdt * ntot, cudaMemcpyDeviceToHost, st));
            ACK(cudaStreamSynchronize(st));
            size_t q = 0;
            for (int i = 0; i < ntot; i++)
                if (alive[i]) {
                    for (size_t w = 0; w < wdt; w++) want[k].host[q * wdt + w] = tmp[(size_t)i * wdt + w];
                    q++;
                }
        }
        if (want_type) {
            std::vector<int32_t> t(ntot);
            ACK(cudaMemcpyAsync(t.data(), stg.type, 4 * (size_t)ntot, cudaMemcpyDeviceToHost, st));
            ACK(cudaStreamSynchronize(st));
            int q = 0;
            for (int i = 0; i < ntot; i++)
                if (dense || alive[i]) o->type[q++] = t[i];
        }
        ACK(cudaStreamSynchronize(st));
        if ((mask & TSPH_ALE_F_INDEX) && o->index) {
            int q = 0;
            for (int i = 0; i < ntot; i++)
                if (dense || alive[i]) o->index[q++] = i;
        }
        return 0;
    }

    // refuse calls that read or write the state while an upload is staged
    int no_staged_upload(std::string &err) const {
        if (!up_pending) return 0;
        err = "an upload is staged: call tsph_ale_particle_to_cell first";
        return TSPH_ERR_STATE;
    }

    int transfer_streams(std::string &err) {
        if (cs_d) return 0;
        ACK(cudaStreamCreateWithFlags(&cs_d, cudaStreamNonBlocking));
        ACK(cudaStreamCreateWithFlags(&cs_u, cudaStreamNonBlocking));
        for (cudaEvent_t *q : {&ev_x, &ev_d, &ev_up, &ev_imp})
            ACK(cudaEventCreateWithFlags(q, cudaEventDisableTiming));
        ACK(cudaEventRecord(ev_imp, st));
        return 0;
    }

    // pipelined download of r, v, rho: exported on the system's stream into
    // a staging set of its own, copied to the host on a copy stream; with
    // removed particles a synchronous download (rows compacted on the host)
    int download_async(int mask, const tsph_ale_host_state *o, std::string &err) {
        int rc;
        if (mask & ~(TSPH_ALE_F_R | TSPH_ALE_F_V | TSPH_ALE_F_RHO)) {
            err = "tsph_ale_download_async: r, v and rho only";
            return TSPH_ERR_ARG;
        }
        // (allowed while an upload is staged: the export reads the state the
        // staged upload changes only when particle_to_cell applies it)
        if ((rc = download_wait(err)) || (rc = normalize(err))) return rc;
        uint32_t nl = 0;
        ACK(cudaMemcpyAsync(&nl, fstart + ncells, 4, cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        if ((long long)nl + nw != (long long)ntot) {
            if (up_pending) {
                err = "tsph_ale_download_async after removals with an upload staged";
                return TSPH_ERR_STATE;
            }
            return download(mask, o, err);
        }
        if ((rc = transfer_streams(err))) return rc;
        AleStage S{};
        struct Want {
            int bit;
            double *host;
            double **dev;
            double **use;
            int width;
        };
        const Want want[] = {{TSPH_ALE_F_R, o->r, &dstg.r, &S.r, 2},
                             {TSPH_ALE_F_V, o->v, &dstg.v, &S.v, 2},
                             {TSPH_ALE_F_RHO, o->rho, &dstg.rho, &S.rho, 1}};
        for (const Want &q : want) {
            if (!(mask & q.bit) || !q.host) continue;
            if ((rc = stage(q.dev, (size_t)q.width, err))) return rc;
            *q.use = *q.dev;
        }
        if ((rc = stage(&dstg.alive, 1, err))) return rc;
        S.alive = dstg.alive;
        k_ale_export<<<nblk(nw + nf), kBlock, 0, st>>>(A, fstart, ncells, W, nw, S, rho0, dp * dp,
                                                       cs * cs * rho0 / 7.);
        ACK(cudaGetLastError());
        ACK(cudaEventRecord(ev_x, st));
        ACK(cudaStreamWaitEvent(cs_d, ev_x, 0));
        for (const Want &q : want)
            if (*q.use)
                ACK(cudaMemcpyAsync(q.host, *q.use, 8 * (size_t)q.width * ntot,
                                    cudaMemcpyDeviceToHost, cs_d));
        ACK(cudaEventRecord(ev_d, cs_d));
        d_pending = true;
        return 0;
    }

    int download_wait(std::string &err) {
        if (!d_pending) return 0;
        d_pending = false;
        ACK(cudaEventSynchronize(ev_d));
        return 0;
    }

    // staged upload of r, v, rho: host-to-device copies on a copy stream
    // beside the work in flight, applied by the next particle_to_cell
    int upload_async(int mask, const tsph_ale_host_state *in, std::string &err) {
        int rc;
        if (mask & ~(TSPH_ALE_F_R | TSPH_ALE_F_V | TSPH_ALE_F_RHO)) {
            err = "tsph_ale_upload_async: r, v and rho only";
            return TSPH_ERR_ARG;
        }
        if ((rc = no_staged_upload(err)) || (rc = transfer_streams(err))) return rc;
        struct Put {
            int bit;
            const double *host;
            double **dev;
            int width;
        };
        const Put put[] = {{TSPH_ALE_F_R, in->r, &ustg.r, 2},
                           {TSPH_ALE_F_V, in->v, &ustg.v, 2},
                           {TSPH_ALE_F_RHO, in->rho, &ustg.rho, 1}};
        // the staging set is free once the last staged import has read it
        ACK(cudaStreamWaitEvent(cs_u, ev_imp, 0));
        int m = 0;
        for (const Put &q : put) {
            if (!(mask & q.bit) || !q.host) continue;
            if ((rc = stage(q.dev, (size_t)q.width, err))) return rc;
            ACK(cudaMemcpyAsync(*q.dev, q.host, 8 * (size_t)q.width * ntot,
                                cudaMemcpyHostToDevice, cs_u));
            m |= q.bit;
        }
        ACK(cudaEventRecord(ev_up, cs_u));
        up_pending = true;
        up_mask = m;
        return 0;
    }

    // upload omega, v, rho and r of fluid particles (omega*v and omega*rho
    // follow), host arrays in the reference's order: staged by index, applied
    // per fluid row on the device (k_ale_import)
    int upload(int mask, const tsph_ale_host_state *in, std::string &err) {
        if (int rc = no_staged_upload(err)) return rc;
        if (int rc = normalize(err)) return rc;
        ACK(cudaStreamSynchronize(st));
        uint32_t nl = 0;
        ACK(cudaMemcpy(&nl, fstart + ncells, 4, cudaMemcpyDeviceToHost));
        if (nl + nw != (uint32_t)ntot) {
            err = "upload after removals is not supported on the ALE path";
            return TSPH_ERR_STATE;
        }
        int rc;
        AleStage S{};
        struct Put {
            int bit;
            const double *host;
            double **dev;
            double **use;
            int width;
        };
        const Put put[] = {{TSPH_ALE_F_OMEGA, in->omega, &stg.om, &S.om, 1},
                           {TSPH_ALE_F_RHO, in->rho, &stg.rho, &S.rho, 1},
                           {TSPH_ALE_F_V, in->v, &stg.v, &S.v, 2},
                           {TSPH_ALE_F_R, in->r, &stg.r, &S.r, 2}};
        for (const Put &q : put) {
            if (!(mask & q.bit) || !q.host) continue;
            if ((rc = stage(q.dev, (size_t)q.width, err))) return rc;
            ACK(cudaMemcpyAsync(*q.dev, q.host, 8 * (size_t)q.width * ntot, cudaMemcpyHostToDevice, st));
            *q.use = *q.dev;
        }
        k_ale_import<<<nblk(nf), kBlock, 0, st>>>(A, fstart, ncells, S, rho0, nw, ntot, nullptr);
        ACK(cudaGetLastError());
        ACK(cudaStreamSynchronize(st));
        if (mask & TSPH_ALE_F_R) cells = false;
        return 0;
    }
};

}  // namespace tsph

struct tsph_ale_system {
    tsph::AleEngine e;
};

namespace {
int afail(int code, const std::string &m) {
    tsph::set_last_error(m);
    return code;
}
int aready(tsph_ale_system *s) {
    if (!s) return afail(TSPH_ERR_ARG, "null system handle");
    if (!s->e.divided) return afail(TSPH_ERR_STATE, "call tsph_ale_divide_to_cells first");
    if (!s->e.built) {
        std::string err;
        int rc = s->e.build(err);
        if (rc) return afail(rc, err);
    }
    return TSPH_OK;
}
int acells(tsph_ale_system *s) {
    if (!s->e.cells) return afail(TSPH_ERR_STATE, "cell lists are stale: call tsph_ale_particle_to_cell");
    return TSPH_OK;
}
}  // namespace

#define AREADY(s)                         \
    do {                                  \
        int rc_ = aready(s);              \
        if (rc_) return rc_;              \
    } while (0)
#define ARUN(expr)                        \
    do {                                  \
        std::string err_;                 \
        int rc_ = (expr);                 \
        if (rc_) return afail(rc_, err_); \
    } while (0)

extern "C" {

int tsph_ale_create(const tsph_constants *c, const tsph_domain *d, void *stream,
                    tsph_ale_system **out) {
    if (!c || !d || !out) return afail(TSPH_ERR_ARG, "null argument");
    *out = nullptr;
    if (!(c->h > 0) || !(c->kap > 0) || !(c->dp > 0) || !(c->cs > 0) || !(c->rho0 > 0))
        return afail(TSPH_ERR_ARG, "h, kap, dp, cs and rho0 must be positive");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return afail(TSPH_ERR_CUDA, "no CUDA device available");
    }
    tsph_ale_system *s = new tsph_ale_system();
    tsph::AleEngine &e = s->e;
    e.h = c->h;
    e.kap = c->kap;
    e.cs = c->cs;
    e.rho0 = c->rho0;
    e.visco = c->visco;
    e.delta = c->delta;
    e.dp = c->dp;
    e.m = c->rho0 / (1 / c->dp * 1 / c->dp);
    e.x0 = d->x_0;
    e.xm = d->x_m;
    e.y0 = d->y_0;
    e.ym = d->y_m;
    if (stream) {
        e.st = static_cast<cudaStream_t>(stream);
    } else {
        if (cudaStreamCreateWithFlags(&e.st, cudaStreamNonBlocking) != cudaSuccess) {
            delete s;
            return afail(TSPH_ERR_CUDA, "cudaStreamCreate failed");
        }
        e.own = true;
    }
    *out = s;
    return TSPH_OK;
}

int tsph_ale_destroy(tsph_ale_system *s) {
    delete s;
    return TSPH_OK;
}

int tsph_ale_add_particles(tsph_ale_system *s, int n, const int32_t *type, const double *r,
                           const double *v, const double *rho, const double *p,
                           const double *normal) {
    if (!s) return afail(TSPH_ERR_ARG, "null system handle");
    if (n < 0 || (n > 0 && (!type || !r || !rho))) return afail(TSPH_ERR_ARG, "bad arguments");
    if (s->e.built) return afail(TSPH_ERR_STATE, "add all particles before the first step");
    for (int i = 0; i < n; i++) {
        if (type[i] != TSPH_FLUID && type[i] != TSPH_WALL)
            return afail(TSPH_ERR_UNSUPPORTED, "only fluid and wall particles are on this path");
        if (type[i] == TSPH_WALL && !normal)
            return afail(TSPH_ERR_ARG, "wall particles of the ALE path need a normal");
        s->e.type.push_back(type[i]);
        s->e.r.push_back(r[2 * i]);
        s->e.r.push_back(r[2 * i + 1]);
        s->e.v.push_back(v ? v[2 * i] : 0.);
        s->e.v.push_back(v ? v[2 * i + 1] : 0.);
        s->e.rho.push_back(rho[i]);
        s->e.p.push_back(p ? p[i] : 0.);
        s->e.nrm.push_back(normal ? normal[2 * i] : 0.);
        s->e.nrm.push_back(normal ? normal[2 * i + 1] : 0.);
    }
    return TSPH_OK;
}

int tsph_ale_set_keep_cells(tsph_ale_system *s, int on) {
    if (!s) return afail(TSPH_ERR_ARG, "null system handle");
    s->e.keep = on != 0;
    return TSPH_OK;
}

int tsph_ale_sort_count(tsph_ale_system *s, long long *n) {
    if (!s || !n) return afail(TSPH_ERR_ARG, "null argument");
    *n = 0;
    if (!s->e.built) return TSPH_OK;
    unsigned long long v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, s->e.sort_runs, 8, cudaMemcpyDeviceToHost, s->e.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->e.st);
    if (e != cudaSuccess) return afail(TSPH_ERR_CUDA, cudaGetErrorString(e));
    *n = (long long)v;
    return TSPH_OK;
}

int tsph_ale_set_scheme(tsph_ale_system *s, int scheme) {
    if (!s) return afail(TSPH_ERR_ARG, "null system handle");
    if (scheme != TSPH_ALE_AS_WRITTEN && scheme != TSPH_ALE_MUSCL && scheme != TSPH_ALE_FIRST_ORDER)
        return afail(TSPH_ERR_ARG, "unknown scheme");
    s->e.scheme = scheme;
    return TSPH_OK;
}

int tsph_ale_np(tsph_ale_system *s, int *np) {
    if (!s || !np) return afail(TSPH_ERR_ARG, "null argument");
    if (!s->e.built) {
        *np = (int)s->e.type.size();
        return TSPH_OK;
    }
    ARUN(s->e.np_live(np, err_));
    return TSPH_OK;
}

int tsph_ale_divide_to_cells(tsph_ale_system *s) {
    if (!s) return afail(TSPH_ERR_ARG, "null system handle");
    tsph::AleEngine &e = s->e;
    const double kh = e.kap * e.h, of = e.h * 0.273;
    const double qx = (e.xm - e.x0 + of) / kh, qy = (e.ym - e.y0 + of) / kh;
    if (!(qx < 1e7) || !(qy < 1e7)) return afail(TSPH_ERR_ARG, "grid too large");
    e.ncx = (int)qx + 1;
    e.ncy = (int)qy + 1;
    if (e.ncy < 4) return afail(TSPH_ERR_UNSUPPORTED, "grid needs at least 4 cells in y");
    e.ncells = e.ncx * e.ncy;
    e.kh = kh;
    e.of = of;
    e.bx.resize(e.ncx + 1);
    e.by.resize(e.ncy + 1);
    for (int k = 0; k <= e.ncx; k++) e.bx[k] = tsph::cell_lower_bound(k, e.x0, of, kh);
    for (int k = 0; k <= e.ncy; k++) e.by[k] = tsph::cell_lower_bound(k, e.y0, of, kh);
    e.ox.resize(e.ncx);
    e.oy.resize(e.ncy);
    for (int k = 0; k < e.ncx; k++) e.ox[k] = (e.x0 - of) + k * kh;
    for (int k = 0; k < e.ncy; k++) e.oy[k] = (e.y0 - of) + k * kh;
    e.divided = true;
    e.built = false;
    return TSPH_OK;
}

int tsph_ale_particle_to_cell(tsph_ale_system *s) {
    AREADY(s);
    ARUN(s->e.particle_to_cell(err_));
    return TSPH_OK;
}

int tsph_ale_gradient(tsph_ale_system *s) {
    AREADY(s);
    int rc = acells(s);
    if (rc) return rc;
    ARUN(s->e.gradient(err_));
    return TSPH_OK;
}

int tsph_ale_forces(tsph_ale_system *s, double dt) {
    AREADY(s);
    (void)dt;  // only enters the cancelled Hancock term of MUSCL_final
    int rc = acells(s);
    if (rc) return rc;
    ARUN(s->e.forces(err_));
    return TSPH_OK;
}

int tsph_ale_leapfrog_one(tsph_ale_system *s, double dt) {
    AREADY(s);
    ARUN(s->e.lf1(dt, err_));
    return TSPH_OK;
}

int tsph_ale_leapfrog_two(tsph_ale_system *s, double dt, int step) {
    AREADY(s);
    ARUN(s->e.lf2(dt, step, err_));
    return TSPH_OK;
}

int tsph_ale_step(tsph_ale_system *s, double dt, int step0, int nsteps) {
    AREADY(s);
    if (nsteps < 0 || step0 < 0) return afail(TSPH_ERR_ARG, "bad step range");
    int rc = acells(s);
    if (rc) return rc;
    ARUN(s->e.step(dt, step0, nsteps, err_));
    return TSPH_OK;
}

int tsph_ale_download(tsph_ale_system *s, int fields, const tsph_ale_host_state *out) {
    AREADY(s);
    if (!out) return afail(TSPH_ERR_ARG, "null output");
    ARUN(s->e.download(fields, out, err_));
    return TSPH_OK;
}

int tsph_ale_upload(tsph_ale_system *s, int fields, const tsph_ale_host_state *in) {
    AREADY(s);
    if (!in) return afail(TSPH_ERR_ARG, "null input");
    ARUN(s->e.upload(fields, in, err_));
    return TSPH_OK;
}

int tsph_ale_download_async(tsph_ale_system *s, int fields, const tsph_ale_host_state *out) {
    AREADY(s);
    if (!out) return afail(TSPH_ERR_ARG, "null output");
    ARUN(s->e.download_async(fields, out, err_));
    return TSPH_OK;
}

int tsph_ale_download_wait(tsph_ale_system *s) {
    AREADY(s);
    ARUN(s->e.download_wait(err_));
    return TSPH_OK;
}

int tsph_ale_upload_async(tsph_ale_system *s, int fields, const tsph_ale_host_state *in) {
    AREADY(s);
    if (!in) return afail(TSPH_ERR_ARG, "null input");
    ARUN(s->e.upload_async(fields, in, err_));
    return TSPH_OK;
}

int tsph_ale_sync(tsph_ale_system *s) {
    if (!s) return afail(TSPH_ERR_ARG, "null system handle");
    if (!s->e.st) return TSPH_OK;
    if (cudaStreamSynchronize(s->e.st) != cudaSuccess) return afail(TSPH_ERR_CUDA, "sync failed");
    return TSPH_OK;
}

int tsph_ale_health(tsph_ale_system *s, uint32_t *flags, int clear) {
    if (!s || !flags) return afail(TSPH_ERR_ARG, "null argument");
    *flags = 0;
    if (!s->e.built) return TSPH_OK;
    if (cudaMemcpyAsync(flags, s->e.health, 4, cudaMemcpyDeviceToHost, s->e.st) != cudaSuccess)
        return afail(TSPH_ERR_CUDA, "health read failed");
    if (clear) cudaMemsetAsync(s->e.health, 0, 4, s->e.st);
    cudaStreamSynchronize(s->e.st);
    return TSPH_OK;
}

}  // extern "C"
