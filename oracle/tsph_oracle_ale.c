/*
 * tsph_oracle_ale.c -- CPU oracle of the Riemann / ALE-SPH step
 * (TEST INFRASTRUCTURE).
 *
 * Restates, in plain C99 double precision and in the reference's operation
 * order, the ALE-SPH path of the reference case cases/ALESPH_dambreakLong/
 * MUSCL.h:80-140: the leap-frog of src/RALESPH_integration.h:10-107, the
 * one-sided gradients of src/_testMUSCL_gradientApprox.h:10-231 and the
 * MUSCL / linearised-Riemann flux loop of src/_testMUSCL_interaction.h:13-324
 * (with src/_testMUSCL_schemes.h and src/ALESPH_riemann_solver.h).  Used only
 * by tests/ and the benchmark's CPU leg.  Pinned bit-for-bit against the
 * reference compiled from its own headers (oracle/ref_harness.cpp).
 *
 * As written in the reference, MUSCL_final adds 0.5 dt/dx (F(W_L) - F(W_L)),
 * i.e. zero, so the interface states are the cell states; the neighbour's
 * state carries the active particle's velocity (_nW = {nrho, nrho*av.x,
 * nrho*av.y}, _testMUSCL_interaction.h:185).  The oracle evaluates all of it
 * literally, including the cancelled flux terms.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "tsph_oracle.h"
#include "tsph_oracle_internal.h"

/* ALESPH_Add_particle, src/SPH_particle_system.h:51-108 */
void orc_ale_add_particle(orc_sys *s, int type, double p, double rho, double rx, double ry,
                          double vx, double vy) {
    orc_add_particle(s, type, p, rho, rx, ry, vx, vy, 0., 0.);
    const int i = s->np - 1;
    const double dp2 = s->dp * s->dp;
    s->ale = 1;
    s->om[i] = dp2;
    s->omvx[i] = vx * dp2;
    s->omvy[i] = vy * dp2;
    s->omr[i] = rho * dp2;
    s->om_o[i] = dp2;
    s->omvx_o[i] = vx * dp2;
    s->omvy_o[i] = vy * dp2;
    s->omr_o[i] = rho * dp2;
}

void orc_ale_set_scheme(orc_sys *s, int scheme) { s->ale_scheme = scheme; }

/* special.n.push_back, src/ALESPH_create.h:719 */
void orc_ale_add_normal(orc_sys *s, double nx, double ny) {
    if (s->nn + 1 > s->ncap) {
        int c = s->ncap ? s->ncap * 2 : 256;
        s->nx = orc_xrealloc(s->nx, sizeof(double) * c);
        s->ny = orc_xrealloc(s->ny, sizeof(double) * c);
        s->ncap = c;
    }
    s->nx[s->nn] = nx;
    s->ny[s->nn] = ny;
    s->nn++;
}

static double *ale_field(const orc_sys *s, int f) {
    switch (f) {
    case 0: return s->om;
    case 1: return s->omr;
    case 2: return s->omvx;
    case 3: return s->omvy;
    case 4: return s->dom;
    case 5: return s->domr;
    case 6: return s->domvx;
    case 7: return s->domvy;
    case 8: return s->om_o;
    case 9: return s->omr_o;
    case 10: return s->omvx_o;
    case 11: return s->omvy_o;
    default:
        if (f >= 12 && f < 24) return s->grad[f - 12];
        return NULL;
    }
}

/* ALE field ids: 0 omega, 1 omega*rho, 2-3 omega*v, 4 domega, 5 d(omega rho),
 * 6-7 d(omega v), 8-11 the leap-frog copies, 12-23 gradients (rhoF xy, vxF xy,
 * vyF xy, rhoB xy, vxB xy, vyB xy) */
void orc_ale_get_field(const orc_sys *s, int f, double *out) {
    const double *p = ale_field(s, f);
    if (p) memcpy(out, p, sizeof(double) * s->np);
}

void orc_ale_set_field(orc_sys *s, int f, const double *in) {
    double *p = ale_field(s, f);
    if (p) memcpy(p, in, sizeof(double) * s->np);
}

/* Kernel_gradient_approx, src/_testMUSCL_gradientApprox.h:10-231: forward
 * (neighbour at larger x) and backward one-sided SPH gradients of rho, vx,
 * vy; BT walls enter through their normals. */
void orc_ale_gradient(orc_sys *s) {
    const int ncy = s->ncy, nc = s->ncells;
    const double h = s->h, m = s->m, dp = s->dp;
    const int *cs = s->cell_start, *cl = s->cell_list;
#pragma omp parallel for
    for (int c = 0; c < nc; c++) {
        const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                           c + ncy,     c - 1 + ncy, c - 1,
                           c - 1 - ncy, c - ncy,     c + 1 - ncy};
        for (int i = cs[c]; i < cs[c + 1]; i++) {
            const int ai = cl[i];
            if (s->type[ai] != ORC_FLUID) continue;
            const double arx = s->rx[ai], ary = s->ry[ai];
            const double avx = s->vx[ai], avy = s->vy[ai];
            const double arho = s->rho[ai];
            double gF[6] = {0, 0, 0, 0, 0, 0}, gB[6] = {0, 0, 0, 0, 0, 0};
            double gamma = 0;
            for (int k = 0; k < 9; k++) {
                const int cc = ac[k];
                if (cc < 0 || cc >= nc) continue;
                for (int n = cs[cc]; n < cs[cc + 1]; n++) {
                    const int ni = cl[n];
                    if (ai == ni) continue;
                    const double nrx = s->rx[ni], nry = s->ry[ni];
                    const double nvx = s->vx[ni], nvy = s->vy[ni];
                    const double nrho = s->rho[ni], nomega = s->om[ni];
                    const double drx = arx - nrx, dry = ary - nry;
                    const double drs = sqrt(pow(drx, 2) + pow(dry, 2));
                    double W, F;
                    orc_wendland(drs, h, &W, &F);
                    const double dWx = drx * F, dWy = dry * F;
                    double *g = NULL;
                    if (nrx > arx) g = gF;
                    else if (nrx < arx) g = gB;
                    if (s->type[ni] == ORC_WALL) {
                        const double nbx = s->nx[ni] * (-1), nby = s->ny[ni] * (-1);
                        if (g) {
                            g[0] += (nrho - arho) * nbx * W * dp;
                            g[1] += (nrho - arho) * nby * W * dp;
                            g[2] += (nvx - avx) * nbx * W * dp;
                            g[3] += (nvx - avx) * nby * W * dp;
                            g[4] += (nvy - avy) * nbx * W * dp;
                            g[5] += (nvy - avy) * nby * W * dp;
                        }
                    } else if (g) {
                        g[0] += (nrho - arho) * nomega * dWx;
                        g[1] += (nrho - arho) * nomega * dWy;
                        g[2] += (nvx - avx) * nomega * dWx;
                        g[3] += (nvx - avx) * nomega * dWy;
                        g[4] += (nvy - avy) * nomega * dWx;
                        g[5] += (nvy - avy) * nomega * dWy;
                    }
                    gamma += W * m / nrho;
                }
            }
            for (int q = 0; q < 6; q++) {
                s->grad[q][ai] = gamma == 0 ? 0. : gF[q] * 2.;
                s->grad[6 + q][ai] = gamma == 0 ? 0. : gB[q] * 2.;
            }
        }
    }
}

/* MUSCL_superBee_L / _R, src/_testMUSCL_schemes.h:33-77 */
static double superbee_D(double gFx, double gFy, double gBx, double gBy, double drx,
                         double dry) {
    const double beta = 2.;
    const double DF = gFx * drx + gFy * dry;
    const double DB = gBx * drx + gBy * dry;
#define MX(a, b) (((a) > (b)) ? (a) : (b))
#define MN(a, b) (((a) < (b)) ? (a) : (b))
    if (DF > 0) return MX(0, MX(MN(beta * DB, DF), MN(DB, DF)));
    if (DF < 0) return MN(0, MN(MX(beta * DB, DF), MX(DB, DF)));
    return 0.;
#undef MX
#undef MN
}

/* F(W, rho0, cs), src/_testMUSCL_schemes.h:18-30 */
static void flux_F(const double W[3], double rho0, double cs, double F[3]) {
    const double p = orc_pressure(W[0], rho0, cs);
    F[0] = W[1] + W[2];
    F[1] = W[1] * W[1] / W[0] + p + W[1] * W[2] / W[0];
    F[2] = W[1] * W[2] / W[0] + W[2] * W[2] / W[0] + p;
}

/* MUSCL_final, src/_testMUSCL_schemes.h:78-88 (as written: the difference of
 * one flux with itself) */
static void muscl_final(const double WaL[3], const double aW[3], double dt, double dx,
                        double rho0, double cs, double W[3]) {
    for (int k = 0; k < 3; k++) {
        double Fa[3], Fb[3];
        flux_F(WaL, rho0, cs, Fa);
        flux_F(WaL, rho0, cs, Fb);
        W[k] = aW[k] + 0.5 * dt / dx * (Fa[k] - Fb[k]);
    }
}

/* Compute_Forces(particles, dt), src/_testMUSCL_interaction.h:13-324 */
void orc_ale_forces(orc_sys *s, double dt) {
    const int ncy = s->ncy, nc = s->ncells;
    const double h = s->h, m = s->m, c0 = s->cs, rho0 = s->rho0, dp = s->dp;
    const double gx = 0., gy = s->gravy;
    const int *cs = s->cell_start, *cl = s->cell_list;
#pragma omp parallel for schedule(dynamic, 3)
    for (int c = 0; c < nc; c++) {
        const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                           c + ncy,     c - 1 + ncy, c - 1,
                           c - 1 - ncy, c - ncy,     c + 1 - ncy};
        /* declared per cell and never reset per particle, :49 */
        double gamma_sum = 0;
        for (int i = cs[c]; i < cs[c + 1]; i++) {
            const int ai = cl[i];
            if (s->type[ai] != ORC_FLUID) continue;
            const double arx = s->rx[ai], ary = s->ry[ai];
            const double avx = s->vx[ai], avy = s->vy[ai];
            const double arho = s->rho[ai];
            const double ao = s->om[ai];
            double gA[12];
            for (int q = 0; q < 12; q++) gA[q] = s->grad[q][ai];
            double dom_s = 0, domr_s = 0, domvx_s = 0, domvy_s = 0;
            for (int k = 0; k < 9; k++) {
                const int cc = ac[k];
                if (cc < 0 || cc >= nc) continue;
                for (int n = cs[cc]; n < cs[cc + 1]; n++) {
                    const int ni = cl[n];
                    if (ai == ni) continue;
                    const double nrx = s->rx[ni], nry = s->ry[ni];
                    const double nvx = s->vx[ni], nvy = s->vy[ni];
                    const double nrho = s->rho[ni];
                    const double no = s->om[ni];
                    double gN[12];
                    for (int q = 0; q < 12; q++) gN[q] = s->grad[q][ni];
                    const double drx = arx - nrx, dry = ary - nry;
                    const double dvx = avx - nvx, dvy = avy - nvy;
                    const double drs = sqrt((drx * drx) + (dry * dry));
                    double W, F;
                    orc_wendland(drs, h, &W, &F);
                    const double dWx = drx * F, dWy = dry * F;
                    const double dvdW = dvx * dWx + dvy * dWy;
                    const double drnx = drx * (1 / drs) * (-1), drny = dry * (1 / drs) * (-1);
                    /* MUSCL reconstructions (gradient order: rhoF, vxF, vyF, rhoB, vxB, vyB) */
                    const double arhoL = arho - superbee_D(gA[0], gA[1], gA[6], gA[7], drx, dry);
                    const double arhoR = arho + superbee_D(gA[0], gA[1], gA[6], gA[7], drx, dry);
                    const double nrhoL = nrho - superbee_D(gN[0], gN[1], gN[6], gN[7], drx, dry);
                    const double nrhoR = nrho + superbee_D(gN[0], gN[1], gN[6], gN[7], drx, dry);
                    const double avLx = avx - superbee_D(gA[2], gA[3], gA[8], gA[9], drx, dry);
                    const double avLy = avy - superbee_D(gA[4], gA[5], gA[10], gA[11], drx, dry);
                    const double avRx = avx + superbee_D(gA[2], gA[3], gA[8], gA[9], drx, dry);
                    const double avRy = avy + superbee_D(gA[4], gA[5], gA[10], gA[11], drx, dry);
                    const double nvLx = nvx - superbee_D(gN[2], gN[3], gN[8], gN[9], drx, dry);
                    const double nvLy = nvy - superbee_D(gN[4], gN[5], gN[10], gN[11], drx, dry);
                    const double nvRx = nvx + superbee_D(gN[2], gN[3], gN[8], gN[9], drx, dry);
                    const double nvRy = nvy + superbee_D(gN[4], gN[5], gN[10], gN[11], drx, dry);
                    (void)arhoR; (void)nrhoL; (void)avRx; (void)avRy; (void)nvLx; (void)nvLy;
                    (void)nrhoR; (void)nvRx; (void)nvRy;
                    const double aW_[3] = {arho, arho * avx, arho * avy};
                    const double nW_[3] = {nrho, nrho * avx, nrho * avy};
                    const double aWL_[3] = {arhoL, arhoL * avLx, arhoL * avLy};
                    const double nWL_[3] = {nrhoL, nrhoL * nvLx, nrhoL * nvLy};
                    double aWL[3], nWR[3];
                    muscl_final(aWL_, aW_, dt, h, rho0, c0, aWL);
                    muscl_final(nWL_, nW_, dt, h, rho0, c0, nWR);
                    double rhoL = aWL[0], rhoR = nWR[0];
                    const double avLx2 = aWL[1] / aWL[0], avLy2 = aWL[2] / aWL[0];
                    const double nvRx2 = nWR[1] / nWR[0], nvRy2 = nWR[2] / nWR[0];
                    double vL = avLx2 * drnx + avLy2 * drny;
                    double vR = nvRx2 * drnx + nvRy2 * drny;
                    if (s->ale_scheme == 1) {
                        /* MUSCL: a extrapolated towards b, b towards a */
                        rhoL = arhoL;
                        rhoR = nrhoR;
                        vL = avLx * drnx + avLy * drny;
                        vR = nvRx * drnx + nvRy * drny;
                    }
                    const double avgc = c0;
                    const double avgrho = 0.5 * (arho + nrho);
                    /* velRiemannLinearized / densRiemannLinearized,
                     * src/ALESPH_riemann_solver.h:6-18,86-96 */
                    const double vss = 0.5 * (vR + vL) - 0.5 * (rhoR - rhoL) * avgc / avgrho;
                    double rhos = 0.5 * (rhoL + rhoR) + 0.5 * (vL - vR) * avgrho / avgc;
                    double ps = orc_pressure(rhos, rho0, c0);
                    const double vsx = drnx * vss + ((avx + nvx) * 0.5 - drnx * (vL + vR) * 0.5);
                    const double vsy = drny * vss + ((avy + nvy) * 0.5 - drny * (vL + vR) * 0.5);
                    const double vzx = avx, vzy = avy;
                    const double vsdW = (vsx - vzx) * dWx + (vsy - vzy) * dWy;
                    if (s->type[ni] == ORC_WALL) {
                        const double nbx = s->nx[ni] * (-1), nby = s->ny[ni] * (-1);
                        rhos = arho - ((0 - avx) * nbx + (0 - avy) * nby) * arho / c0;
                        ps = orc_pressure(rhos, rho0, c0) * 1;
                        domvx_s -= 2 * W * dp * (ps * nbx);
                        domvy_s -= 2 * W * dp * (ps * nby);
                    } else {
                        domvx_s -= 2 * no *
                                   ((rhos * vsx * (vsx - vzx) + ps) * dWx + (rhos * vsx * (vsy - vzy)) * dWy);
                        domvy_s -= 2 * no *
                                   ((rhos * vsy * (vsx - vzx)) * dWx + (rhos * vsy * (vsy - vzy) + ps) * dWy);
                    }
                    if (s->type[ni] == ORC_WALL) {
                        const double nbx = s->nx[ni] * (-1), nby = s->ny[ni] * (-1);
                        const double dvn = dvx * nbx + dvy * nby;
                        dom_s -= dvn * W * dp;
                    } else {
                        dom_s -= dvdW * no;
                        domr_s -= 2 * rhos * no * vsdW;
                    }
                    gamma_sum += W * m / nrho;
                }
            }
            if (gamma_sum == 0) {
                s->dom[ai] = 0.;
                s->domr[ai] = 0.;
                s->domvx[ai] = 0.;
                s->domvy[ai] = 0.;
            } else {
                s->dom[ai] = dom_s * ao;
                s->domr[ai] = domr_s * ao;
                s->domvx[ai] = domvx_s * ao - gx * ao * arho;
                s->domvy[ai] = domvy_s * ao - gy * ao * arho;
            }
        }
    }
}

/* Compute_Forces(Particle_system&), src/RALESPH_interaction.h:12-289: the
 * first-order variant of cases/ALESPH_dambreakLong/SPH_simulationINT.h (both
 * particles' own states, velRiemannLinearized and
 * densRiemannLinearizedWithLimiter, src/ALESPH_riemann_solver.h:20-34,86-96;
 * BT walls with the linear equation of state Compute_Pressure2,
 * src/SPH_pressure.h:24-34) */
void orc_ale_forces_first_order(orc_sys *s) {
    const int ncy = s->ncy, nc = s->ncells;
    const double h = s->h, m = s->m, c0 = s->cs, rho0 = s->rho0, dp = s->dp;
    const double gx = 0., gy = s->gravy;
    const int *cs = s->cell_start, *cl = s->cell_list;
#pragma omp parallel for schedule(dynamic, 3)
    for (int c = 0; c < nc; c++) {
        const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                           c + ncy,     c - 1 + ncy, c - 1,
                           c - 1 - ncy, c - ncy,     c + 1 - ncy};
        double gamma_sum = 0; /* per cell, never reset per particle */
        for (int i = cs[c]; i < cs[c + 1]; i++) {
            const int ai = cl[i];
            if (s->type[ai] != ORC_FLUID) continue;
            const double arx = s->rx[ai], ary = s->ry[ai];
            const double avx = s->vx[ai], avy = s->vy[ai];
            const double arho = s->rho[ai];
            const double ao = s->om[ai];
            double dom_s = 0, domr_s = 0, domvx_s = 0, domvy_s = 0;
            for (int k = 0; k < 9; k++) {
                const int cc = ac[k];
                if (cc < 0 || cc >= nc) continue;
                for (int n = cs[cc]; n < cs[cc + 1]; n++) {
                    const int ni = cl[n];
                    if (ai == ni) continue;
                    const double nvx = s->vx[ni], nvy = s->vy[ni];
                    const double nrho = s->rho[ni];
                    const double no = s->om[ni];
                    const double drx = arx - s->rx[ni], dry = ary - s->ry[ni];
                    const double dvx = avx - nvx, dvy = avy - nvy;
                    const double drs = sqrt((drx * drx) + (dry * dry));
                    double W, F;
                    orc_wendland(drs, h, &W, &F);
                    const double dWx = drx * F, dWy = dry * F;
                    const double dvdW = dvx * dWx + dvy * dWy;
                    const double drnx = drx * (1 / drs) * (-1), drny = dry * (1 / drs) * (-1);
                    const double vL = avx * drnx + avy * drny;
                    const double vR = nvx * drnx + nvy * drny;
                    const double avgrho = 0.5 * (arho + nrho);
                    const double vss = 0.5 * (vR + vL) - 0.5 * (nrho - arho) * c0 / avgrho;
                    const double d = vL - vR;
                    const double mx = (d > 0) ? d : 0;
                    const double beta = ((3. * mx) < c0) ? (3. * mx) : c0;
                    double rhos = 0.5 * (arho + nrho) + 0.5 * beta * (vL - vR) * avgrho / (c0 * c0);
                    double ps = orc_pressure(rhos, rho0, c0);
                    const double vsx = drnx * vss + ((avx + nvx) * 0.5 - drnx * (vL + vR) * 0.5);
                    const double vsy = drny * vss + ((avy + nvy) * 0.5 - drny * (vL + vR) * 0.5);
                    const double vzx = avx, vzy = avy;
                    if (s->type[ni] == ORC_WALL) {
                        const double nbx = s->nx[ni] * (-1), nby = s->ny[ni] * (-1);
                        rhos = arho - ((0 - avx) * nbx + (0 - avy) * nby) * arho / c0;
                        ps = c0 * c0 * (rhos - rho0) * 1;
                        domvx_s -= 2 * W * dp * (ps * nbx);
                        domvy_s -= 2 * W * dp * (ps * nby);
                        const double dvn = dvx * nbx + dvy * nby;
                        dom_s -= dvn * W * dp;
                    } else {
                        domvx_s -= 2 * no *
                                   ((rhos * vsx * (vsx - vzx) + ps) * dWx + (rhos * vsx * (vsy - vzy)) * dWy);
                        domvy_s -= 2 * no *
                                   ((rhos * vsy * (vsx - vzx)) * dWx + (rhos * vsy * (vsy - vzy) + ps) * dWy);
                        const double vsdW = (vsx - vzx) * dWx + (vsy - vzy) * dWy;
                        dom_s -= dvdW * no;
                        domr_s -= 2 * rhos * no * vsdW;
                    }
                    gamma_sum += W * m / nrho;
                }
            }
            if (gamma_sum == 0) {
                s->dom[ai] = 0.;
                s->domr[ai] = 0.;
                s->domvx[ai] = 0.;
                s->domvy[ai] = 0.;
            } else {
                s->dom[ai] = dom_s * ao;
                s->domr[ai] = domr_s * ao;
                s->domvx[ai] = domvx_s * ao - gx * ao * arho;
                s->domvy[ai] = domvy_s * ao - gy * ao * arho;
            }
        }
    }
}

/* Integrate_LeapFrog_partOne, src/RALESPH_integration.h:10-36 */
void orc_ale_leapfrog_one(orc_sys *s, double dt) {
#pragma omp parallel for schedule(static)
    for (int p = 0; p < s->np; p++) {
        if (s->type[p] != ORC_FLUID) continue;
        s->om_o[p] = s->om[p];
        s->omr_o[p] = s->omr[p];
        s->omvx_o[p] = s->omvx[p];
        s->omvy_o[p] = s->omvy[p];
        s->om[p] = s->om[p] + s->dom[p] * dt * 0.5;
        s->omr[p] = s->omr[p] + s->domr[p] * dt * 0.5;
        s->omvx[p] = s->omvx[p] + s->domvx[p] * dt * 0.5;
        s->omvy[p] = s->omvy[p] + s->domvy[p] * dt * 0.5;
        s->rho[p] = s->omr[p] / (s->om[p]);
        s->vx[p] = s->omvx[p] / (s->rho[p] * s->om[p]);
        s->vy[p] = s->omvy[p] / (s->rho[p] * s->om[p]);
    }
    s->cells_built = s->cells_built; /* positions unchanged */
}

/* Integrate_LeapFrog_partTwo, src/RALESPH_integration.h:38-107 */
void orc_ale_leapfrog_two(orc_sys *s, double dt, int step) {
    if (step == 1) {
#pragma omp parallel for schedule(static)
        for (int p = 0; p < s->np; p++) {
            if (s->type[p] != ORC_FLUID) continue;
            s->om_o[p] = s->om[p];
            s->omr_o[p] = s->omr[p];
            s->omvx_o[p] = s->omvx[p];
            s->omvy_o[p] = s->omvy[p];
            s->om[p] = s->om[p] + s->dom[p] * dt * 0.5;
            s->omr[p] = s->omr[p] + s->domr[p] * dt * 0.5;
            s->omvx[p] = s->omvx[p] + s->domvx[p] * dt * 0.5;
            s->omvy[p] = s->omvy[p] + s->domvy[p] * dt * 0.5;
            s->rho[p] = s->omr[p] / (s->om[p]);
            s->vx[p] = s->omvx[p] / (s->rho[p] * s->om[p]);
            s->vy[p] = s->omvy[p] / (s->rho[p] * s->om[p]);
            s->rx[p] = s->rx[p] + s->vx[p] * dt * 0.5;
            s->ry[p] = s->ry[p] + s->vy[p] * dt * 0.5;
        }
    } else {
#pragma omp parallel for schedule(static)
        for (int p = 0; p < s->np; p++) {
            if (s->type[p] != ORC_FLUID) continue;
            s->rx[p] = s->rx[p] + s->vx[p] * dt;
            s->ry[p] = s->ry[p] + s->vy[p] * dt;
            s->om[p] = s->om_o[p] + s->dom[p] * dt;
            s->omr[p] = s->omr_o[p] + s->domr[p] * dt;
            s->omvx[p] = s->omvx_o[p] + s->domvx[p] * dt;
            s->omvy[p] = s->omvy_o[p] + s->domvy[p] * dt;
            s->rho[p] = s->omr[p] / (s->om[p]);
            s->vx[p] = s->omvx[p] / (s->rho[p] * s->om[p]);
            s->vy[p] = s->omvy[p] / (s->rho[p] * s->om[p]);
        }
    }
    s->cells_built = 0;
}

/* One body of SPH_simulation::RUN of cases/ALESPH_dambreakLong/MUSCL.h:82-137
 * per step, steps step0+1 .. step0+nsteps.  Particles leaving the domain are
 * removed consistently from every array (the case calls the non-ALE remover,
 * which leaves special.* misaligned, src/SPH_btdebug.h:4-31 vs :33-58). */
void orc_ale_step(orc_sys *s, double dt, int step0, int nsteps) {
    for (int k = 1; k <= nsteps; k++) {
        const int step = step0 + k;
        if (step > 1) orc_ale_leapfrog_one(s, dt);
        orc_clear_cells(s);
        orc_particle_to_cell(s);
        orc_density_to_pressure(s);
        if (s->ale_scheme == 2) {
            orc_ale_forces_first_order(s); /* SPH_simulationINT.h: no gradient pass */
        } else {
            orc_ale_gradient(s);
            orc_ale_forces(s, dt);
        }
        orc_ale_leapfrog_two(s, dt, step);
        orc_remove_out_of_domain(s);
    }
}
