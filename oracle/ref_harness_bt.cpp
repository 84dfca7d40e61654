// ref_harness_bt.cpp -- C entry points around the UNMODIFIED reference
// headers of the boundary-integral (BT) WCSPH path (TEST INFRASTRUCTURE).
//
// Built by oracle/Makefile (target `ref`) from the reference's src/ into
// oracle/_ref/libtsph_ref_bt.so.  A translation unit of its own because
// src/SPH_interactionBT.h defines Compute_Forces(Particle_system&) beside the
// other flavours.  Calls the functions of
// cases/damBreakLong_BT/SPH_simulationSymplectic.h in its RUN order, and of
// cases/flowDrop_BT/SPH_simulationSymplectic.h (the same with buffer zones).

#include "SPH_defs.h"
#include "SPH_particle_system.h"
#include "SPH_find_pairs.h"
#include "SPH_pressure.h"
#include "SPH_interactionBT.h"
#include "SPH_integration.h"
#include "ALESPH_create.h"
#include "SPH_BT.h"
#include "SPH_btdebug.h"
#include "SPH_inlet_outlet_data.h"
#include "SPH_buffer_zones.h"

#include <iostream>
#include <sstream>

namespace {
struct RefCase {
    Particle_system particles;
    Simulation_data sim;
    RefCase(double h, double kap, double cs, double rho0, double visco, double delta, double dp,
            double x0, double xm, double y0, double ym)
        : particles(h, kap, cs, rho0, visco, delta, dp), sim(x0, xm, y0, ym) {
        sim.hh = h;
        sim.kh = h * kap;
        sim.nvl = 0;
    }
};
struct Quiet {
    std::streambuf *old;
    std::ostringstream sink;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet() { std::cout.rdbuf(old); }
};
RefCase *K(void *c) { return static_cast<RefCase *>(c); }
}  // namespace

extern "C" {

void *refbt_create(double h, double kap, double cs, double rho0, double visco, double delta,
                   double dp, double x0, double xm, double y0, double ym) {
    return new RefCase(h, kap, cs, rho0, visco, delta, dp, x0, xm, y0, ym);
}
void refbt_destroy(void *c) { delete K(c); }
void refbt_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}
void refbt_add_particle(void *c, int type, double p, double rho, double rx, double ry, double vx,
                        double vy) {
    K(c)->particles.ALESPH_Add_particle((unsigned short)type, p, rho, TDouble2(rx, ry),
                                        TDouble2(vx, vy), TDouble2(0., 0.));
}
void refbt_add_normal(void *c, double nx, double ny) {
    K(c)->particles.special.n.push_back(TDouble2(nx, ny));
}
// generators of src/ALESPH_create.h (cases/damBreakLong_BT/geometry.h)
void refbt_create_wall_x_bt(void *c, double x0, double x1, double y, int o, double nx, double ny) {
    Create_Wall_x_bt(K(c)->particles, x0, x1, y, o, TDouble2(nx, ny));
}
void refbt_create_wall_y_bt(void *c, double x, double y0, double y1, int o, double nx, double ny) {
    Create_Wall_y_bt(K(c)->particles, x, y0, y1, o, TDouble2(nx, ny));
}
void refbt_create_corner_bt(void *c, int ox, int oy, double xv, double yv, double nx, double ny) {
    Create_corner_bt(K(c)->particles, ox, oy, TDouble2(xv, yv), TDouble2(nx, ny));
}
void refbt_create_block_of_fluid_wp(void *c, double x0, double y0, double x1, double y1) {
    Quiet q;
    Create_Block_of_FluidWP(K(c)->particles, x0, y0, x1, y1);
}
int refbt_np(void *c) { return (int)K(c)->particles.np; }
int refbt_nn(void *c) { return (int)K(c)->particles.special.n.size(); }
void refbt_get_normals(void *c, double *n) {
    for (size_t i = 0; i < K(c)->particles.special.n.size(); i++) {
        n[2 * i] = K(c)->particles.special.n[i].x;
        n[2 * i + 1] = K(c)->particles.special.n[i].y;
    }
}
// state in particle order: r, v, a (2n), rho, drho, p (n), type, index
void refbt_get_state(void *c, double *r, double *v, double *a, double *rho, double *drho,
                     double *p, int *type, int *index) {
    Particle_system &P = K(c)->particles;
    for (unsigned i = 0; i < P.np; i++) {
        if (r) { r[2 * i] = P.data.r[i].x; r[2 * i + 1] = P.data.r[i].y; }
        if (v) { v[2 * i] = P.data.v[i].x; v[2 * i + 1] = P.data.v[i].y; }
        if (a) { a[2 * i] = P.data.a[i].x; a[2 * i + 1] = P.data.a[i].y; }
        if (rho) rho[i] = P.data.rho[i];
        if (drho) drho[i] = P.data.drho[i];
        if (p) p[i] = P.data.p[i];
        if (type) type[i] = P.data.part_type[i];
        if (index) index[i] = P.data.index[i];
    }
}
void refbt_set_velocity_density(void *c, const double *v, const double *rho) {
    Particle_system &P = K(c)->particles;
    for (unsigned i = 0; i < P.np; i++) {
        if (P.data.part_type[i] != fluid) continue;
        P.data.v[i] = TDouble2(v[2 * i], v[2 * i + 1]);
        P.data.rho[i] = rho[i];
    }
}
void refbt_divide_to_cells(void *c) {
    Quiet q;
    Divide_To_Cells(K(c)->particles, K(c)->sim);
}
void refbt_particle_to_cell(void *c) {
    Clear_cells(K(c)->particles);
    Particle_To_Cell(K(c)->particles, K(c)->sim);
}
void refbt_density_to_pressure(void *c) {
    Quiet q;
    Density_to_pressure(K(c)->particles);
}
void refbt_wall_density(void *c) {
    Quiet q;
    BT_compute_density_BTGeo(K(c)->particles, K(c)->sim);
}
void refbt_forces(void *c) {
    Quiet q;
    Compute_Forces(K(c)->particles);
}
// the body of SPH_simulation::RUN of cases/damBreakLong_BT/SPH_simulationSymplectic.h
void refbt_step(void *c, double dt, int n) {
    Quiet q;
    Particle_system &P = K(c)->particles;
    for (int k = 0; k < n; k++) {
        BT_compute_density_BTGeo(P, K(c)->sim);
        Density_to_pressure(P);
        Integrate_SymplecticPredictor(P, dt);
        Clear_cells(P);
        Particle_To_Cell(P, K(c)->sim);
        Density_to_pressure(P);
        Compute_Forces(P);
        Integrate_SymplecticCorrector(P, dt);
        RemoveParticlesOutOfDomain(P, K(c)->sim);
        Clear_cells(P);
        Particle_To_Cell(P, K(c)->sim);
        Density_to_pressure(P);
        Compute_Forces(P);
    }
}

// buffer zones (the BufferZone constructor of src/SPH_inlet_outlet_data.h)
void refbt_add_zone(void *c, double x0, double xm, double y0, double ym, int nbl, double vx,
                    double vy, double ox, double oy, int btype) {
    K(c)->particles.zones.push_back(
        BufferZone(x0, xm, y0, ym, nbl, TDouble2(vx, vy), TDouble2(ox, oy), btype));
}
void refbt_create_inlet_x(void *c, double y, double x0, double x1, int o, int nbl, double vx,
                          double vy, int type) {
    Quiet q;
    DRAW_CreateInletX(K(c)->particles, y, x0, x1, o, nbl, TDouble2(vx, vy), type);
}
void refbt_create_outlet_y(void *c, double x, double y0, double y1, int o, int nbl, double vx,
                           double vy, int type, int empty) {
    Quiet q;
    DRAW_CreateOutletY(K(c)->particles, x, y0, y1, o, nbl, TDouble2(vx, vy), type, empty != 0);
}
// the body of SPH_simulation::RUN of cases/flowDrop_BT/SPH_simulationSymplectic.h
void refbt_step_zones(void *c, double dt, int n) {
    Quiet q;
    Particle_system &P = K(c)->particles;
    for (int k = 0; k < n; k++) {
        BT_compute_density_BTGeo(P, K(c)->sim);
        Density_to_pressure(P);
        Integrate_SymplecticPredictor(P, dt);
        for (int z = 0; z < (int)P.zones.size(); z++) {  // inlets, then outlets, by zone
            if (P.zones[z].btype >= outlet) BZ_Integrate_outlet(P, z, dt);
            else BZ_Integrate_inlet(P, z, dt);
        }
        Clear_cells(P);
        Particle_To_Cell(P, K(c)->sim);
        Density_to_pressure(P);
        Compute_Forces(P);
        Integrate_SymplecticCorrector(P, dt);
        RemoveParticlesOutOfDomain(P, K(c)->sim);
        Clear_cells(P);
        Particle_To_Cell(P, K(c)->sim);
        Density_to_pressure(P);
        Compute_Forces(P);
    }
}

}  // extern "C"
