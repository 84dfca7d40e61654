/*
 * tsph_oracle_zones.c -- open boundaries of the oracle (TEST INFRASTRUCTURE):
 * inlet and outlet buffer zones, src/SPH_buffer_zones.h and
 * src/SPH_inlet_outlet_data.h, restated in C.  Buffer particles keep their
 * type (the zone's btype) until they cross the zone line; they are
 * neighbours of the fluid but not force targets (src/SPH_interaction.h
 * skips non-fluid rows), are left out of the mDBC sums (fluid only,
 * src/SPH_kernel_approx.h:1246) and of RemoveParticlesOutOfDomain (fluid
 * only), and are integrated by the symplectic scheme like every particle.
 */
#include <math.h>
#include <string.h>

#include "tsph_oracle.h"
#include "tsph_oracle_internal.h"

int orc_add_zone(orc_sys *s, double x0, double xm, double y0, double ym, int nbl, double vx,
                 double vy, double ox, double oy, int btype) {
    if (s->nzones >= ORC_MAX_ZONES) return -1;
    orc_zone *z = &s->zones[s->nzones];
    z->x0 = x0; z->xm = xm; z->y0 = y0; z->ym = ym;
    z->nbl = nbl; z->vbx = vx; z->vby = vy; z->ox = ox; z->oy = oy; z->btype = btype;
    /* BufferZone constructor, src/SPH_inlet_outlet_data.h */
    z->bl = fabs(xm - x0);
    z->bh = fabs(ym - y0);
    if (ox != 0) { z->bl = fabs(xm - x0); z->bh = fabs(ym - y0); }
    else if (oy != 0) { z->bl = fabs(ym - y0); z->bh = fabs(xm - x0); }
    return s->nzones++;
}

/* Add_particle(type, 0, 1000, r, v_b, {0, 0}), src/SPH_particle_system.h:25-50 */
static void add_buffer_particle(orc_sys *s, int type, double rx, double ry, double vx, double vy) {
    orc_add_particle(s, type, 0., 1000., rx, ry, vx, vy, 0., 0.);
}

/* BZ_Integrate_inlet, src/SPH_buffer_zones.h:10-108.  The loop runs over
 * the particles present when it starts (np is re-read each iteration in the
 * reference, so particles appended in this call are visited too; they lie
 * on the inner side of the zone line and do not cross it). */
void orc_bz_inlet(orc_sys *s, int zone, double dt) {
    const orc_zone Z = s->zones[zone];
    double x_b = 0;
    int orientation = 0;
    if (Z.ox != 0) { x_b = Z.x0; orientation = (int)Z.ox; }
    else if (Z.oy != 0) { x_b = Z.y0; orientation = (int)Z.oy; }
    const double b_len = Z.bl;
    const int t = Z.btype;
    if (Z.ox != 0) {
        if (orientation < 0) {
            for (int p = 0; p < s->np; p++) {
                if (s->type[p] != t) continue;
                if (s->rx[p] > x_b) {
                    s->type[p] = ORC_FLUID;
                    add_buffer_particle(s, t, s->rx[p] - b_len, s->ry[p], Z.vbx, Z.vby);
                }
            }
        } else if (orientation > 0) {
            for (int p = 0; p < s->np; p++) {
                if (s->type[p] != t) continue;
                s->rx[p] = s->rx[p] + s->vx[p] * dt;
                if (s->rx[p] < x_b) {
                    s->type[p] = ORC_FLUID;
                    add_buffer_particle(s, t, s->rx[p] + b_len, s->ry[p], Z.vbx, Z.vby);
                }
            }
        }
    } else if (Z.oy != 0) {
        for (int p = 0; p < s->np; p++) {
            if (s->type[p] != t) continue;
            s->ry[p] = s->ry[p] + s->vy[p] * dt;
            if (orientation < 0 ? (s->ry[p] > x_b) : (s->ry[p] < x_b)) {
                s->type[p] = ORC_FLUID;
                add_buffer_particle(s, t, s->rx[p], orientation < 0 ? s->ry[p] - b_len
                                                                    : s->ry[p] + b_len,
                                    Z.vbx, Z.vby);
            }
        }
    }
    s->cells_built = 0;
}

/* BZ_Integrate_outlet, src/SPH_buffer_zones.h:111-206 (x orientation; the
 * reference's y branches are empty).  Remove_particle erases inside the
 * forward loop, so the particle that slides into slot p is not examined in
 * that call; the same happens here. */
void orc_bz_outlet(orc_sys *s, int zone, double dt) {
    (void)dt;
    const orc_zone Z = s->zones[zone];
    if (Z.ox == 0) return;
    const double dp = s->dp;
    const double x_b = Z.x0, b_len = Z.bl;
    const int orientation = (int)Z.ox, t = Z.btype;
    for (int p = 0; p < s->np; p++) {
        if (s->type[p] == ORC_FLUID) {
            if (orientation > 0 ? (s->rx[p] > x_b) : (s->rx[p] < x_b)) {
                s->type[p] = t;
                s->ax[p] = 0.;
                s->ay[p] = 0.;
                s->drho[p] = 0.;
            }
        } else if (s->type[p] == t) {
            const int out = orientation > 0 ? (s->rx[p] > x_b + b_len) : (s->rx[p] < x_b - b_len);
            if (out || s->ry[p] < dp / 2) orc_erase_particle(s, p);
        }
    }
    s->cells_built = 0;
}

/* The RUN body of the cases with buffer zones (cases/inflowSlab_mDBC,
 * cases/flowDrop_mDBC with mDBC walls, cases/flowDrop_BT with
 * boundary-integral walls: BT_compute_density_BTGeo and the BT
 * Compute_Forces), every zone's inlet or outlet after the predictor. */
void orc_step_zones(orc_sys *s, int model, double dt, int nsteps) {
    for (int k = 0; k < nsteps; k++) {
        if (model == ORC_BT) orc_bt_density(s);
        else orc_mdbc_density(s);
        orc_density_to_pressure(s);
        orc_predictor(s, dt);
        for (int z = 0; z < s->nzones; z++) {  /* the cases call inlets, then outlets, by zone */
            if (s->zones[z].btype >= 11) orc_bz_outlet(s, z, dt);
            else orc_bz_inlet(s, z, dt);
        }
        orc_clear_cells(s);
        orc_particle_to_cell(s);
        orc_density_to_pressure(s);
        orc_compute_forces(s, model);
        orc_corrector(s, dt);
        orc_remove_out_of_domain(s);
        orc_clear_cells(s);
        orc_particle_to_cell(s);
        orc_density_to_pressure(s);
        orc_compute_forces(s, model);
    }
}
