// ref_harness_ale.cpp -- C entry points around the UNMODIFIED reference
// headers of the ALE-SPH path (TEST INFRASTRUCTURE).
//
// Built by oracle/Makefile (target `ref`) from the reference's src/ into
// oracle/_ref/libtsph_ref_ale.so.  A translation unit of its own because the
// ALE headers redefine functions of the WCSPH ones (e.g. Integrate_Verlet in
// src/RALESPH_integration.h and src/SPH_integration.h).  Calls the
// functions of cases/ALESPH_dambreakLong/MUSCL.h in its RUN order.

#include "SPH_defs.h"
#include "SPH_particle_system.h"
#include "SPH_find_pairs.h"
#include "SPH_pressure.h"
#include "RALESPH_integration.h"
#include "ALESPH_create.h"
#include "_testMUSCL_gradientApprox.h"
#include "_testMUSCL_interaction.h"
#include "RALESPH_interaction.h"
#include "SPH_btdebug.h"

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

void *refale_create(double h, double kap, double cs, double rho0, double visco, double delta,
                    double dp, double x0, double xm, double y0, double ym) {
    return new RefCase(h, kap, cs, rho0, visco, delta, dp, x0, xm, y0, ym);
}
void refale_destroy(void *c) { delete K(c); }
void refale_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}
void refale_add_particle(void *c, int type, double p, double rho, double rx, double ry, double vx,
                         double vy) {
    K(c)->particles.ALESPH_Add_particle((unsigned short)type, p, rho, TDouble2(rx, ry),
                                        TDouble2(vx, vy), TDouble2(0., 0.));
}
void refale_add_normal(void *c, double nx, double ny) {
    K(c)->particles.special.n.push_back(TDouble2(nx, ny));
}
// generators of src/ALESPH_create.h
void refale_create_wall_x_bt(void *c, double x0, double x1, double y, int o, double nx, double ny) {
    Create_Wall_x_bt(K(c)->particles, x0, x1, y, o, TDouble2(nx, ny));
}
void refale_create_wall_y_bt(void *c, double x, double y0, double y1, int o, double nx, double ny) {
    Create_Wall_y_bt(K(c)->particles, x, y0, y1, o, TDouble2(nx, ny));
}
void refale_create_corner_bt(void *c, int ox, int oy, double xv, double yv, double nx, double ny) {
    Create_corner_bt(K(c)->particles, ox, oy, TDouble2(xv, yv), TDouble2(nx, ny));
}
void refale_create_block_of_fluid(void *c, double x0, double y0, double x1, double y1) {
    Quiet q;
    Create_Block_of_Fluid(K(c)->particles, x0, y0, x1, y1);
}
int refale_np(void *c) { return (int)K(c)->particles.np; }
int refale_nn(void *c) { return (int)K(c)->particles.special.n.size(); }
void refale_get_normals(void *c, double *n) {
    for (size_t i = 0; i < K(c)->particles.special.n.size(); i++) {
        n[2 * i] = K(c)->particles.special.n[i].x;
        n[2 * i + 1] = K(c)->particles.special.n[i].y;
    }
}
// state: r, v (2n), rho, p (n), type, index; ALE: omega, omegarho, omegav (2n),
// domega, domegarho, domegav (2n), gradients (12n: rhoF vxF vyF rhoB vxB vyB)
void refale_get_state(void *c, double *r, double *v, double *rho, double *p, int *type,
                      int *index, double *om, double *omr, double *omv, double *dom,
                      double *domr, double *domv, double *grad) {
    Particle_system &P = K(c)->particles;
    for (unsigned i = 0; i < P.np; i++) {
        if (r) { r[2 * i] = P.data.r[i].x; r[2 * i + 1] = P.data.r[i].y; }
        if (v) { v[2 * i] = P.data.v[i].x; v[2 * i + 1] = P.data.v[i].y; }
        if (rho) rho[i] = P.data.rho[i];
        if (p) p[i] = P.data.p[i];
        if (type) type[i] = P.data.part_type[i];
        if (index) index[i] = P.data.index[i];
        if (om) om[i] = P.special.omega[i];
        if (omr) omr[i] = P.special.omegarho[i];
        if (omv) { omv[2 * i] = P.special.omegav[i].x; omv[2 * i + 1] = P.special.omegav[i].y; }
        if (dom) dom[i] = P.special.domega[i];
        if (domr) domr[i] = P.special.domegarho[i];
        if (domv) { domv[2 * i] = P.special.domegav[i].x; domv[2 * i + 1] = P.special.domegav[i].y; }
        if (grad) {
            const tdouble2 g[6] = {P.special.gradrhoF[i], P.special.gradvxF[i], P.special.gradvyF[i],
                                   P.special.gradrhoB[i], P.special.gradvxB[i], P.special.gradvyB[i]};
            for (int k = 0; k < 6; k++) {
                grad[12 * i + 2 * k] = g[k].x;
                grad[12 * i + 2 * k + 1] = g[k].y;
            }
        }
    }
}
void refale_set_velocity_density(void *c, const double *v, const double *rho) {
    // consistent ALE state: v, rho and omega*v, omega*rho (omega unchanged)
    Particle_system &P = K(c)->particles;
    for (unsigned i = 0; i < P.np; i++) {
        if (P.data.part_type[i] != fluid) continue;
        P.data.v[i] = TDouble2(v[2 * i], v[2 * i + 1]);
        P.data.rho[i] = rho[i];
        P.special.omegav[i] = P.data.v[i] * P.special.omega[i];
        P.special.omegarho[i] = rho[i] * P.special.omega[i];
    }
}
void refale_divide_to_cells(void *c) {
    Quiet q;
    Divide_To_Cells(K(c)->particles, K(c)->sim);
}
void refale_particle_to_cell(void *c) {
    Clear_cells(K(c)->particles);
    Particle_To_Cell(K(c)->particles, K(c)->sim);
}
void refale_density_to_pressure(void *c) {
    Quiet q;
    Density_to_pressure(K(c)->particles);
}
void refale_gradient(void *c) { Kernel_gradient_approx(K(c)->particles); }
void refale_forces(void *c, double dt) {
    Quiet q;
    Compute_Forces(K(c)->particles, dt);
}
void refale_leapfrog_one(void *c, double dt) { Integrate_LeapFrog_partOne(K(c)->particles, dt); }
void refale_leapfrog_two(void *c, double dt, int step) {
    Integrate_LeapFrog_partTwo(K(c)->particles, dt, step);
}
// The body of SPH_simulation::RUN of cases/ALESPH_dambreakLong/MUSCL.h:85-130
// for steps step0+1 .. step0+n (with the ALE remover, which keeps the special
// arrays aligned with the particle arrays).
void refale_step(void *c, double dt, int step0, int n) {
    Quiet q;
    Particle_system &P = K(c)->particles;
    for (int k = 1; k <= n; k++) {
        const int step = step0 + k;
        if (step > 1) Integrate_LeapFrog_partOne(P, dt);
        Clear_cells(P);
        Particle_To_Cell(P, K(c)->sim);
        Density_to_pressure(P);
        Kernel_gradient_approx(P);
        Compute_Forces(P, dt);
        Integrate_LeapFrog_partTwo(P, dt, step);
        RemoveParticlesOutOfDomain_ALE(P, K(c)->sim);
    }
}

// the first-order variant of cases/ALESPH_dambreakLong/SPH_simulationINT.h:84-133
// (Compute_Forces(Particle_system&), src/RALESPH_interaction.h:12-289; no
// gradient pass)
void refale_forces_first_order(void *c) { Compute_Forces(K(c)->particles); }

void refale_step_first_order(void *c, double dt, int step0, int n) {
    Quiet q;
    Particle_system &P = K(c)->particles;
    for (int k = 1; k <= n; k++) {
        const int step = step0 + k;
        if (step > 1) Integrate_LeapFrog_partOne(P, dt);
        Clear_cells(P);
        Particle_To_Cell(P, K(c)->sim);
        Density_to_pressure(P);
        Compute_Forces(P);
        Integrate_LeapFrog_partTwo(P, dt, step);
        RemoveParticlesOutOfDomain_ALE(P, K(c)->sim);
    }
}

}  // extern "C"
