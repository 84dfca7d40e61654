// tsph_zones.cuh -- open boundaries on the device: inlet and outlet buffer
// zones, src/SPH_buffer_zones.h:10-206 (BufferZone of
// src/SPH_inlet_outlet_data.h).  Buffer particles are fluid rows whose type
// is the zone's; the reference's particle order (creation order, erasures
// closing the gaps) is the order of particle indices here, so every
// order-dependent rule is evaluated on indices.
#pragma once

#include "tsph_kernels.cuh"

namespace tsph {

struct ZoneDev {
    double ox, oy;        // orientation
    double x_b;           // zone line (x0 for x zones, y0 for y zones)
    double b_len;         // buffer length
    double vbx, vby;      // buffer velocity
    int btype;            // type of the zone's buffer particles
    double dp;
};

// BZ_Integrate_inlet, first half: buffer particles of the zone move (all
// branches but the x, orientation < 0 one, which the reference leaves to
// the integrator) and those past the zone line turn into fluid; each such
// parent is listed (its index, its row) for the appends
template <typename T>
__global__ void k_inlet_cross(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                              ZoneDev Z, double dt, uint32_t *__restrict__ list, int cap,
                              uint32_t *__restrict__ count) {
    pdl_enter();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_live(fstart, ncells)) return;
    if (F.key[f] == (uint32_t)ncells || F.type[f] != (uint8_t)Z.btype) return;
    double2 r = F.r[f];
    const auto v = F.v[f];
    bool cross;
    if (Z.ox != 0) {
        if (Z.ox < 0) {
            cross = r.x > Z.x_b;
        } else {
            r.x = r.x + (double)v.x * dt;
            cross = r.x < Z.x_b;
        }
    } else {
        r.y = r.y + (double)v.y * dt;
        cross = Z.oy < 0 ? (r.y > Z.x_b) : (r.y < Z.x_b);
    }
    F.r[f] = r;
    if (!cross) return;
    F.type[f] = 0;
    const uint32_t k = atomicAdd(count, 1u);
    if ((int)k < cap) {
        list[2 * k] = F.id[f];
        list[2 * k + 1] = (uint32_t)f;
    }
}

// BZ_Integrate_inlet, second half: Add_particle(btype, 0, 1000, r -+ b_len,
// v_b, 0) for every listed parent, in the order of the parents' indices
// (the reference appends while it walks its arrays): the new particle gets
// index next_id + rank and row n_live + rank, its old state equals its
// state (src/SPH_particle_system.h:25-50)
// (the reference's loop reaches the appended particles too: in the branches
// that move buffer particles they move by v_b dt in the same call, their
// old position staying where they were created)
template <typename T>
__global__ void k_inlet_append(FluidState<T> F, OldState<T> O, const uint32_t *__restrict__ fstart,
                               int ncells, ZoneDev Z, const uint32_t *__restrict__ list, int k,
                               uint32_t next_id, T rho0, double dt) {
    pdl_enter();
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= k) return;
    const uint32_t pid = list[2 * e];
    const int prow = (int)list[2 * e + 1];
    int rank = 0;
    for (int q = 0; q < k; q++) rank += list[2 * q] < pid ? 1 : 0;
    const int row = (int)fstart[ncells] + rank;
    const double2 pr = F.r[prow];
    double2 r = pr;
    if (Z.ox != 0) r.x = Z.ox < 0 ? pr.x - Z.b_len : pr.x + Z.b_len;
    else r.y = Z.oy < 0 ? pr.y - Z.b_len : pr.y + Z.b_len;
    typename V2<T>::t v, zero;
    v.x = (T)Z.vbx;
    v.y = (T)Z.vby;
    zero.x = T(0);
    zero.y = T(0);
    const T rho = rho_stored_from_full<T>(1000.0, (double)rho0);
    double2 rm = r;
    if (Z.ox > 0) rm.x = r.x + (double)v.x * dt;
    else if (Z.ox == 0) rm.y = r.y + (double)v.y * dt;
    F.r[row] = rm;
    F.v[row] = v;
    F.a[row] = zero;
    F.rho[row] = rho;
    F.drho[row] = T(0);
    F.p[row] = T(0);
    F.id[row] = next_id + (uint32_t)rank;
    F.key[row] = 0u;  // live, cell assigned by the next binning
    F.loc[row] = make_float2(0.f, 0.f);
    F.type[row] = (uint8_t)Z.btype;
    O.r[row] = r;
    O.v[row] = v;
    O.rho[row] = rho;
}

// the appended rows join the live range
static __global__ void k_grow_live(uint32_t *__restrict__ fstart, int ncells, int k) {
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        fstart[ncells] += (uint32_t)k;
        fstart[ncells + 1] += (uint32_t)k;
    }
}

// BZ_Integrate_outlet (x zones), first pass: which indices are present
// (walls included: they are in the reference's arrays) and which buffer
// particles of the zone are to be erased (past the far side of the buffer,
// or below dp / 2)
template <typename T>
__global__ void k_outlet_mark(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                              const uint32_t *__restrict__ wid, int nw, ZoneDev Z,
                              uint8_t *__restrict__ live, uint8_t *__restrict__ cand) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        live[wid[i]] = 1;
        return;
    }
    const int f = i - nw;
    if (f >= n_live(fstart, ncells) || F.key[f] == (uint32_t)ncells) return;
    const uint32_t id = F.id[f];
    live[id] = 1;
    if (F.type[f] != (uint8_t)Z.btype) return;
    const double2 r = F.r[f];
    const bool out = Z.ox > 0 ? (r.x > Z.x_b + Z.b_len) : (r.x < Z.x_b - Z.b_len);
    if (out || r.y < Z.dp / 2) cand[id] = 1;
}

// the reference erases inside forward loops (Remove_particle / erase), so
// the particle right after an erased one is not examined in that call: with
// `live` the indices present and `cand` the erase candidates, a particle is
// skipped when the run of candidates just before it (in index order, over
// present indices) has odd length
__device__ __forceinline__ bool skipped_after_erase(const uint8_t *__restrict__ live,
                                                    const uint8_t *__restrict__ cand, int id) {
    int c = 0;
    for (int j = id - 1; j >= 0; j--) {
        if (!live[j]) continue;
        if (!cand[j]) break;
        c++;
    }
    return (c & 1) != 0;
}

// RemoveParticlesOutOfDomain, src/SPH_btdebug.h:4-31, first pass: present
// indices (walls included) and the fluid outside the padded box
template <typename T>
__global__ void k_remove_mark(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                              const uint32_t *__restrict__ wid, int nw, Box box,
                              uint8_t *__restrict__ live, uint8_t *__restrict__ cand) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nw) {
        live[wid[i]] = 1;
        return;
    }
    const int f = i - nw;
    if (f >= n_live(fstart, ncells) || F.key[f] == (uint32_t)ncells) return;
    const uint32_t id = F.id[f];
    live[id] = 1;
    if (F.type && F.type[f] != 0) return;  // fluid only (src/SPH_btdebug.h:18)
    if (out_of_domain(F.r[f], box)) cand[id] = 1;
}

// second pass: a candidate is erased unless the erase of the particle before
// it skipped it
template <typename T>
__global__ void k_remove_apply(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                               const uint8_t *__restrict__ live, const uint8_t *__restrict__ cand,
                               uint32_t *__restrict__ removed, uint32_t *__restrict__ health,
                               uint8_t *__restrict__ dead) {
    pdl_enter();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_live(fstart, ncells) || F.key[f] == (uint32_t)ncells) return;
    const int id = (int)F.id[f];
    if (!cand[id] || skipped_after_erase(live, cand, id)) return;
    F.key[f] = (uint32_t)ncells;
    if (dead) dead[id] = 1;
    atomicAdd(removed, 1u);
    atomicOr(health, kHealthRemoved);
}

// BZ_Integrate_outlet, second pass.  The reference erases inside its forward loop, so the
// particle right after an erased one is not examined in that call: a
// particle is skipped when the run of erase candidates just before it (in
// index order, over present indices) has odd length; otherwise fluid past
// the zone line becomes a buffer particle (a = 0, drho = 0) and an erase
// candidate is removed
template <typename T>
__global__ void k_outlet_apply(FluidState<T> F, const uint32_t *__restrict__ fstart, int ncells,
                               ZoneDev Z, const uint8_t *__restrict__ live,
                               const uint8_t *__restrict__ cand, uint32_t *__restrict__ removed,
                               uint32_t *__restrict__ health) {
    pdl_enter();
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_live(fstart, ncells) || F.key[f] == (uint32_t)ncells) return;
    const int id = (int)F.id[f];
    if (skipped_after_erase(live, cand, id)) return;
    if (F.type[f] == 0) {
        const double2 r = F.r[f];
        if (Z.ox > 0 ? (r.x > Z.x_b) : (r.x < Z.x_b)) {
            F.type[f] = (uint8_t)Z.btype;
            typename V2<T>::t zero;
            zero.x = T(0);
            zero.y = T(0);
            F.a[f] = zero;
            F.drho[f] = T(0);
        }
    } else if (cand[id]) {
        F.key[f] = (uint32_t)ncells;
        atomicAdd(removed, 1u);
        atomicOr(health, kHealthRemoved);
    }
}

}  // namespace tsph
