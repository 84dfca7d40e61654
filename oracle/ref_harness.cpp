// ref_harness.cpp -- C entry points around the UNMODIFIED reference headers
// (TEST INFRASTRUCTURE).
//
// Built by oracle/Makefile (target `ref`) straight from the reference's own
// src/ directory (-I <reference>/src) into oracle/_ref/libtsph_ref.so with the
// reference's own compiler flags (src/Makefile:25).  Nothing of the reference
// is copied here: this file only includes its headers and calls its
// functions, in the order its case drivers call them.  It exists to pin the
// plain-C oracle (oracle/tsph_oracle.c) bit-for-bit and to generate the
// golden vectors under tests/golden/.  x86-64 only in practice: the
// reference sources are not present where the GPU runs.
//
// Both pair-loop flavours define `void Compute_Forces(Particle_system&)`
// (src/SPH_interaction.h:8 and src/SPH_interactionDBC.h:8); the second one is
// renamed with a macro so both can live in one translation unit.

#include "SPH_defs.h"
#include "SPH_particle_system.h"
#include "SPH_find_pairs.h"
#include "SPH_pressure.h"
#include "SPH_interaction.h"
#define Compute_Forces Compute_Forces_DBC
#include "SPH_interactionDBC.h"
#undef Compute_Forces
#include "SPH_integration.h"
#include "SPH_mDBC.h"
#include "SPH_btdebug.h"
#include "SPH_create.h"
#include "SPH_water_level.h"
#include "SPH_measure_pressure.h"
#include "SPH_inlet_outlet_data.h"
#include "SPH_buffer_zones.h"

#include <iostream>
#include <sstream>

namespace {

struct RefCase {
    Particle_system particles;
    Simulation_data sim;
    RefCase(double h, double kap, double cs, double rho0, double visco,
            double delta, double dp, double x0, double xm, double y0,
            double ym)
        : particles(h, kap, cs, rho0, visco, delta, dp), sim(x0, xm, y0, ym) {
        sim.hh = h;
        sim.kh = h * kap;
        sim.nvl = 0;
    }
};

// The reference prints progress and warnings on std::cout; keep the harness
// quiet by pointing cout at a sink for the duration of a call.
struct Quiet {
    std::streambuf *old;
    std::ostringstream sink;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet() { std::cout.rdbuf(old); }
};

}  // namespace

extern "C" {

void *ref_create(double h, double kap, double cs, double rho0, double visco,
                 double delta, double dp, double x0, double xm, double y0,
                 double ym) {
    return new RefCase(h, kap, cs, rho0, visco, delta, dp, x0, xm, y0, ym);
}

void ref_destroy(void *c) { delete static_cast<RefCase *>(c); }

void ref_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}

void ref_add_particle(void *c, int type, double p, double rho, double rx,
                      double ry, double vx, double vy) {
    RefCase *k = static_cast<RefCase *>(c);
    k->particles.Add_particle((unsigned short)type, p, rho, TDouble2(rx, ry),
                              TDouble2(vx, vy), TDouble2(0., 0.));
}

void ref_add_gnr(void *c, double gx, double gy) {
    static_cast<RefCase *>(c)->particles.special.gnr.push_back(TDouble2(gx, gy));
}

// geometry generators of the reference (src/SPH_create.h)
void ref_create_block_of_fluid(void *c, double x0, double y0, double x1, double y1) {
    Quiet q;
    Create_Block_of_Fluid(static_cast<RefCase *>(c)->particles, x0, y0, x1, y1);
}
void ref_create_block_of_fluid_wp(void *c, double x0, double y0, double x1, double y1) {
    Quiet q;
    Create_Block_of_FluidWP(static_cast<RefCase *>(c)->particles, x0, y0, x1, y1);
}
void ref_create_wall_x_mdbc(void *c, double x0, double x1, double y, int o, double yw) {
    Create_Wall_x_mdbc(static_cast<RefCase *>(c)->particles, x0, x1, y, o, yw);
}
void ref_create_wall_y_mdbc(void *c, double x, double y0, double y1, int o, double xw) {
    Create_Wall_y_mdbc(static_cast<RefCase *>(c)->particles, x, y0, y1, o, xw);
}
void ref_create_corner_mdbc(void *c, int ox, int oy, double xv, double yv) {
    Create_corner_mdbc(static_cast<RefCase *>(c)->particles, ox, oy, TDouble2(xv, yv));
}
void ref_create_wall_x(void *c, double x0, double x1, double y, int o) {
    Create_Wall_x(static_cast<RefCase *>(c)->particles, x0, x1, y, o);
}
void ref_create_wall_y(void *c, double x, double y0, double y1, int o) {
    Create_Wall_y(static_cast<RefCase *>(c)->particles, x, y0, y1, o);
}

// Wendland_kernel, src/SPH_kernel.h:52-77 (returns through its static buffer)
void ref_wendland(double r, double h, double *w, double *f) {
    double *k = Wendland_kernel(r, h);
    *w = k[0];
    *f = k[1];
}

int ref_np(void *c) { return (int)static_cast<RefCase *>(c)->particles.np; }

void ref_grid(void *c, int *ncx, int *ncy) {
    RefCase *k = static_cast<RefCase *>(c);
    *ncx = (int)k->particles.pairs.ncx;
    *ncy = (int)k->particles.pairs.ncy;
}

// state in the reference's particle order
void ref_get_state(void *c, double *r, double *v, double *a, double *rho,
                   double *drho, double *p, int *index, int *type) {
    RefCase *k = static_cast<RefCase *>(c);
    SPH_data &d = k->particles.data;
    for (unsigned i = 0; i < k->particles.np; i++) {
        if (r) { r[2 * i] = d.r[i].x; r[2 * i + 1] = d.r[i].y; }
        if (v) { v[2 * i] = d.v[i].x; v[2 * i + 1] = d.v[i].y; }
        if (a) { a[2 * i] = d.a[i].x; a[2 * i + 1] = d.a[i].y; }
        if (rho) rho[i] = d.rho[i];
        if (drho) drho[i] = d.drho[i];
        if (p) p[i] = d.p[i];
        if (index) index[i] = d.index[i];
        if (type) type[i] = d.part_type[i];
    }
}

void ref_get_gnr(void *c, double *g) {
    RefCase *k = static_cast<RefCase *>(c);
    for (size_t i = 0; i < k->particles.special.gnr.size(); i++) {
        g[2 * i] = k->particles.special.gnr[i].x;
        g[2 * i + 1] = k->particles.special.gnr[i].y;
    }
}

int ref_ngnr(void *c) { return (int)static_cast<RefCase *>(c)->particles.special.gnr.size(); }

// overwrite a state field (same layout as ref_get_state); used to feed the
// reference and the oracle the same perturbed states
void ref_set_state(void *c, const double *r, const double *v, const double *a,
                   const double *rho, const double *drho, const double *p) {
    RefCase *k = static_cast<RefCase *>(c);
    SPH_data &d = k->particles.data;
    for (unsigned i = 0; i < k->particles.np; i++) {
        if (r) { d.r[i].x = r[2 * i]; d.r[i].y = r[2 * i + 1]; }
        if (v) { d.v[i].x = v[2 * i]; d.v[i].y = v[2 * i + 1]; }
        if (a) { d.a[i].x = a[2 * i]; d.a[i].y = a[2 * i + 1]; }
        if (rho) d.rho[i] = rho[i];
        if (drho) d.drho[i] = drho[i];
        if (p) d.p[i] = p[i];
    }
}

// cells[c].cp as CSR; returns the total count
int ref_get_cells(void *c, int *cell_start, int *cell_list) {
    RefCase *k = static_cast<RefCase *>(c);
    int acc = 0;
    for (size_t cc = 0; cc < k->particles.cells.size(); cc++) {
        if (cell_start) cell_start[cc] = acc;
        for (size_t i = 0; i < k->particles.cells[cc].cp.size(); i++) {
            if (cell_list) cell_list[acc] = k->particles.cells[cc].cp[i];
            acc++;
        }
    }
    if (cell_start) cell_start[k->particles.cells.size()] = acc;
    return acc;
}

void ref_divide_to_cells(void *c) {
    Quiet q;
    RefCase *k = static_cast<RefCase *>(c);
    Divide_To_Cells(k->particles, k->sim);
}
void ref_clear_cells(void *c) { Clear_cells(static_cast<RefCase *>(c)->particles); }
void ref_particle_to_cell(void *c) {
    RefCase *k = static_cast<RefCase *>(c);
    Particle_To_Cell(k->particles, k->sim);
}
void ref_density_to_pressure(void *c) {
    Quiet q;
    Density_to_pressure(static_cast<RefCase *>(c)->particles);
}
void ref_compute_forces(void *c, int model) {
    RefCase *k = static_cast<RefCase *>(c);
    if (model == 0)
        Compute_Forces(k->particles);
    else
        Compute_Forces_DBC(k->particles);
}
void ref_mdbc_density(void *c) {
    Quiet q;
    RefCase *k = static_cast<RefCase *>(c);
    mDBC_compute_density_mdbcGeo(k->particles, k->sim);
}
void ref_predictor(void *c, double dt) {
    Integrate_SymplecticPredictor(static_cast<RefCase *>(c)->particles, dt);
}
void ref_corrector(void *c, double dt) {
    Integrate_SymplecticCorrector(static_cast<RefCase *>(c)->particles, dt);
}
void ref_remove_out_of_domain(void *c) {
    Quiet q;
    RefCase *k = static_cast<RefCase *>(c);
    RemoveParticlesOutOfDomain(k->particles, k->sim);
}

// The body of SPH_simulation::RUN: cases/damBreakLong_mDBC/
// SPH_simulationSymplectic.h:64-116 (model 0) and cases/stillWater_DBC/
// SPH_simulationSymplectic.h:68-116 (model 1), without the output blocks.
void ref_step(void *c, int model, double dt, int nsteps) {
    Quiet q;
    RefCase *k = static_cast<RefCase *>(c);
    Particle_system &P = k->particles;
    for (int s = 0; s < nsteps; s++) {
        if (model == 0) {
            mDBC_compute_density_mdbcGeo(P, k->sim);
            Density_to_pressure(P);
        }
        Integrate_SymplecticPredictor(P, dt);
        Clear_cells(P);
        Particle_To_Cell(P, k->sim);
        Density_to_pressure(P);
        if (model == 0) Compute_Forces(P); else Compute_Forces_DBC(P);
        Integrate_SymplecticCorrector(P, dt);
        RemoveParticlesOutOfDomain(P, k->sim);
        Clear_cells(P);
        Particle_To_Cell(P, k->sim);
        Density_to_pressure(P);
        if (model == 0) Compute_Forces(P); else Compute_Forces_DBC(P);
    }
}


// probes of the case drivers (cases/damBreakLong_mDBC/SPH_simulationSymplectic.h:156-199)
double ref_water_level(void *c, double x, double y0, int inverse) {
    RefCase *rc = static_cast<RefCase *>(c);
    Quiet q;
    return inverse ? Water_Elevation_inverse(rc->particles, rc->sim, x, y0)
                   : Water_Elevation(rc->particles, rc->sim, x, y0);
}

void ref_point_fields(void *c, double x, double y, double *out4) {
    RefCase *rc = static_cast<RefCase *>(c);
    const std::array<real, 4> f = Kernel_velocity_approximation_TEST(rc->particles, rc->sim, {x, y});
    for (int k = 0; k < 4; k++) out4[k] = f[k];
}

double ref_pressure_in_point(void *c, double x, double y) {
    RefCase *rc = static_cast<RefCase *>(c);
    return Pressure_in_point(rc->particles, rc->sim, {x, y});
}
// open boundaries (cases/inflowSlab_mDBC): the zone generators of
// src/SPH_create.h, BZ_Integrate_inlet / _outlet and the case's RUN loop
void ref_create_inlet_y(void *c, double x, double y0, double y1, int o, int nbl, double vx,
                        double vy, int type) {
    Quiet q;
    DRAW_CreateInletY(static_cast<RefCase *>(c)->particles, x, y0, y1, o, nbl, TDouble2(vx, vy),
                      type);
}
void ref_create_inlet_x(void *c, double y, double x0, double x1, int o, int nbl, double vx,
                        double vy, int type) {
    Quiet q;
    DRAW_CreateInletX(static_cast<RefCase *>(c)->particles, y, x0, x1, o, nbl, TDouble2(vx, vy),
                      type);
}
void ref_create_outlet_y(void *c, double x, double y0, double y1, int o, int nbl, double vx,
                         double vy, int type, int empty) {
    Quiet q;
    DRAW_CreateOutletY(static_cast<RefCase *>(c)->particles, x, y0, y1, o, nbl, TDouble2(vx, vy),
                       type, empty != 0);
}
void ref_add_zone(void *c, double x0, double xm, double y0, double ym, int nbl, double vx, double vy,
                  double ox, double oy, int btype) {
    static_cast<RefCase *>(c)->particles.zones.push_back(
        BufferZone(x0, xm, y0, ym, nbl, TDouble2(vx, vy), TDouble2(ox, oy), btype));
}
int ref_nzones(void *c) { return (int)static_cast<RefCase *>(c)->particles.zones.size(); }
// orientation x, y; x0, y0, xm, ym; nbl; bl, bh; btype; v_b x, y
void ref_get_zone(void *c, int k, double *out12) {
    const BufferZone &z = static_cast<RefCase *>(c)->particles.zones[k];
    const double v[12] = {z.orientation.x, z.orientation.y, z.x0, z.y0, z.xm, z.ym,
                          (double)z.nbl, z.bl, z.bh, (double)z.btype, z.v_b.x, z.v_b.y};
    for (int i = 0; i < 12; i++) out12[i] = v[i];
}
void ref_bz_inlet(void *c, int zone, double dt) {
    Quiet q;
    BZ_Integrate_inlet(static_cast<RefCase *>(c)->particles, zone, dt);
}
void ref_bz_outlet(void *c, int zone, double dt) {
    Quiet q;
    BZ_Integrate_outlet(static_cast<RefCase *>(c)->particles, zone, dt);
}
// the body of SPH_simulation::RUN of cases/inflowSlab_mDBC and
// cases/flowDrop_mDBC SPH_simulationSymplectic.h
void ref_step_zones(void *c, double dt, int nsteps) {
    Quiet q;
    RefCase *K = static_cast<RefCase *>(c);
    Particle_system &P = K->particles;
    for (int k = 0; k < nsteps; k++) {
        mDBC_compute_density_mdbcGeo(P, K->sim);
        Density_to_pressure(P);
        Integrate_SymplecticPredictor(P, dt);
        for (int z = 0; z < (int)P.zones.size(); z++) {  // inlets, then outlets, by zone
            if (P.zones[z].btype >= outlet) BZ_Integrate_outlet(P, z, dt);
            else BZ_Integrate_inlet(P, z, dt);
        }
        Clear_cells(P);
        Particle_To_Cell(P, K->sim);
        Density_to_pressure(P);
        Compute_Forces(P);
        Integrate_SymplecticCorrector(P, dt);
        RemoveParticlesOutOfDomain(P, K->sim);
        Clear_cells(P);
        Particle_To_Cell(P, K->sim);
        Density_to_pressure(P);
        Compute_Forces(P);
    }
}

}  // extern "C"
