/*
 * tsph_oracle.c -- CPU oracle for the 2D WCSPH time step (TEST INFRASTRUCTURE).
 *
 * Not the product.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library, and only as the checker / the timed CPU
 * baseline.  It restates the reference's algorithm (tomashalada/tinySPH_old,
 * headers under src/) in plain C99 + OpenMP, double precision, keeping the reference's
 * operation order so that a one-thread run is bit-identical to the reference
 * compiled from its own sources.  Compile with -ffp-contract=off: a fused
 * multiply-add would change the last bit relative to the reference (which is
 * built for x86-64 without FMA).
 *
 * Parity pin: tests/test_oracle_golden.py checks this file against vectors
 * produced by the reference itself (oracle/ref_harness.cpp, built from the
 * reference headers by oracle/Makefile).
 *
 * Deliberate deviations from the reference (documented, none on the pinned
 * cases): (1) Wendland_kernel returns through a function-static buffer in the
 * reference (src/SPH_kernel.h:54), a data race under OpenMP; here it returns
 * through locals, so multi-threaded runs are deterministic and equal the
 * one-thread run.  (2) Neighbour cell ids >= ncells are skipped (the
 * reference only checks < 0, src/SPH_interaction.h:74, and would read past
 * the cell vector).  (3) Particles whose cell lies outside the grid are
 * counted as escaped and not binned (the reference indexes out of range).
 */
#include "tsph_oracle.h"
#include "tsph_oracle_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void *orc_xrealloc(void *p, size_t n) {
    void *q = realloc(p, n ? n : 1);
    if (!q) abort();
    return q;
}

void orc_grow(orc_sys *s, int need) {
    if (need <= s->cap) return;
    int c = s->cap ? s->cap : 256;
    while (c < need) c *= 2;
    s->index = orc_xrealloc(s->index, sizeof(int) * c);
    s->type = orc_xrealloc(s->type, sizeof(int) * c);
#define G(f) s->f = orc_xrealloc(s->f, sizeof(double) * c)
    G(p); G(rho); G(drho); G(rx); G(ry); G(vx); G(vy); G(ax); G(ay);
    G(rox); G(roy); G(vox); G(voy); G(rho_o);
    G(om); G(omr); G(omvx); G(omvy); G(om_o); G(omr_o); G(omvx_o); G(omvy_o);
    G(dom); G(domr); G(domvx); G(domvy);
    for (int k = 0; k < 12; k++) s->grad[k] = orc_xrealloc(s->grad[k], sizeof(double) * c);
#undef G
    s->cap = c;
}

/* Particle_system constructor, src/SPH_particle_system.h:191-212;
 * Simulation_data, src/SPH_data.h:121-122 (domain already padded by the
 * caller as in PREP_SIMULATION_DATA). */
orc_sys *orc_create(double h, double kap, double cs, double rho0, double visco,
                    double delta, double dp, double x0, double xm, double y0,
                    double ym) {
    orc_sys *s = calloc(1, sizeof(orc_sys));
    if (!s) abort();
    s->h = h;
    s->kap = kap;
    s->cs = cs;
    s->rho0 = rho0;
    s->dp = dp;
    s->gravy = 9.81;
    s->m = rho0 / (1 / dp * 1 / dp); /* same expression tree as :207 */
    s->avisc = visco;
    s->delta = delta;
    s->x0 = x0;
    s->xm = xm;
    s->y0 = y0;
    s->ym = ym;
    return s;
}

void orc_destroy(orc_sys *s) {
    if (!s) return;
    free(s->index); free(s->type);
    free(s->p); free(s->rho); free(s->drho); free(s->rx); free(s->ry);
    free(s->vx); free(s->vy); free(s->ax); free(s->ay); free(s->rox);
    free(s->roy); free(s->vox); free(s->voy); free(s->rho_o);
    free(s->gx); free(s->gy);
    free(s->om); free(s->omr); free(s->omvx); free(s->omvy); free(s->om_o); free(s->omr_o);
    free(s->omvx_o); free(s->omvy_o); free(s->dom); free(s->domr); free(s->domvx);
    free(s->domvy); free(s->nx); free(s->ny);
    for (int k = 0; k < 12; k++) free(s->grad[k]);
    free(s->cell_start); free(s->cell_list); free(s->cell_count);
    free(s);
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Add_particle, src/SPH_particle_system.h:25-50 */
void orc_add_particle(orc_sys *s, int type, double p, double rho, double rx,
                      double ry, double vx, double vy, double ax, double ay) {
    orc_grow(s, s->np + 1);
    int i = s->np++;
    s->type[i] = type;
    s->index[i] = i;
    s->p[i] = p;
    s->rho[i] = rho;
    s->drho[i] = 0.;
    s->rx[i] = rx; s->ry[i] = ry;
    s->vx[i] = vx; s->vy[i] = vy;
    s->ax[i] = ax; s->ay[i] = ay;
    s->rox[i] = rx; s->roy[i] = ry;
    s->vox[i] = vx; s->voy[i] = vy;
    s->rho_o[i] = rho;
    s->om[i] = s->omr[i] = s->omvx[i] = s->omvy[i] = 0.;
    s->om_o[i] = s->omr_o[i] = s->omvx_o[i] = s->omvy_o[i] = 0.;
    s->dom[i] = s->domr[i] = s->domvx[i] = s->domvy[i] = 0.;
    for (int k = 0; k < 12; k++) s->grad[k][i] = 0.;
    s->cells_built = 0;
}

/* special.gnr.push_back, e.g. src/SPH_create.h:575-577 */
void orc_add_gnr(orc_sys *s, double gx, double gy) {
    if (s->ngnr + 1 > s->gcap) {
        int c = s->gcap ? s->gcap * 2 : 256;
        s->gx = orc_xrealloc(s->gx, sizeof(double) * c);
        s->gy = orc_xrealloc(s->gy, sizeof(double) * c);
        s->gcap = c;
    }
    s->gx[s->ngnr] = gx;
    s->gy[s->ngnr] = gy;
    s->ngnr++;
}

int orc_np(const orc_sys *s) { return s->np; }

void orc_grid(const orc_sys *s, int *ncx, int *ncy) {
    *ncx = s->ncx;
    *ncy = s->ncy;
}

double orc_const(const orc_sys *s, int which) {
    switch (which) {
    case 0: return s->h;
    case 1: return s->kap;
    case 2: return s->dp;
    case 3: return s->cs;
    case 4: return s->rho0;
    case 5: return s->avisc;
    case 6: return s->delta;
    case 7: return s->m;
    case 8: return s->gravy;
    default: return 0.;
    }
}

static double *field_ptr(const orc_sys *s, int f) {
    switch (f) {
    case ORC_F_RX: return s->rx;
    case ORC_F_RY: return s->ry;
    case ORC_F_VX: return s->vx;
    case ORC_F_VY: return s->vy;
    case ORC_F_AX: return s->ax;
    case ORC_F_AY: return s->ay;
    case ORC_F_RHO: return s->rho;
    case ORC_F_DRHO: return s->drho;
    case ORC_F_P: return s->p;
    case ORC_F_ROX: return s->rox;
    case ORC_F_ROY: return s->roy;
    case ORC_F_VOX: return s->vox;
    case ORC_F_VOY: return s->voy;
    case ORC_F_RHO_O: return s->rho_o;
    default: return NULL;
    }
}

void orc_get_field(const orc_sys *s, int field, double *out) {
    const double *p = field_ptr(s, field);
    if (p) memcpy(out, p, sizeof(double) * s->np);
}

void orc_set_field(orc_sys *s, int field, const double *in) {
    double *p = field_ptr(s, field);
    if (p) memcpy(p, in, sizeof(double) * s->np);
    if (field == ORC_F_RX || field == ORC_F_RY) s->cells_built = 0;
}

void orc_get_meta(const orc_sys *s, int *index, int *type) {
    if (index) memcpy(index, s->index, sizeof(int) * s->np);
    if (type) memcpy(type, s->type, sizeof(int) * s->np);
}

int orc_get_cells(const orc_sys *s, int *cell_start, int *cell_list) {
    if (!s->cells_built) return -1;
    memcpy(cell_start, s->cell_start, sizeof(int) * (s->ncells + 1));
    memcpy(cell_list, s->cell_list, sizeof(int) * s->cell_start[s->ncells]);
    return s->cell_start[s->ncells];
}

/* ---------------------------------------------------------------- kernels */

/* Wendland_kernel, src/SPH_kernel.h:52-77.  The reference rounds the two
 * normalisation constants and the (1 - q/2) powers through float; the same
 * conversions happen here so the result is bit-identical. */
void orc_wendland(double r, double h, double *w, double *f) {
    const double awen = (float)(0.557 / (h * h));
    const double bwen = (float)(-2.7852 / (h * h * h));
    const double qq = r / h;
    const float wqq1 = 1.f - 0.5f * qq;
    const float wqq2 = wqq1 * wqq1;
    const float wqq = qq + qq + 1.f;
    double W, F;
    if (qq <= 2.0) {
        W = awen * wqq * wqq2 * wqq2;
        F = bwen * qq * wqq2 * wqq1 / r;
    } else {
        W = 0.0;
        F = 0.0;
    }
    if (r == 0.0) {
        W = awen;
        F = 0.0;
    }
    *w = W;
    *f = F;
}

/* Compute_Pressure (Tait, gamma = 7), src/SPH_pressure.h:7-21 */
double orc_pressure(double rho, double rho0, double c0) {
    const double gamma = 7.;
    const double b_const = c0 * c0 * rho0 / gamma;
    const double rho_r = rho / rho0;
    return b_const * (pow(rho_r, gamma) - 1);
}

/* Pressure_to_density, src/SPH_pressure.h:37-51 */
double orc_pressure_to_density(double p, double rho0, double c0) {
    const double gamma = 7.;
    const double b_const = c0 * c0 * rho0 / gamma;
    (void)gamma;
    return (pow(p / b_const + 1, 1. / 7)) * rho0;
}

/* Artificial_Viscosity, src/SPH_viscouse_forces.h:7-25 */
static inline double av_term(double h, double drs, double drdv, double rho0,
                             double c0, double alpha) {
    double av = 0;
    const double visco = drdv > alpha ? drdv : alpha;
    if (drdv < 0) {
        const double mu = h * drdv / (drs * drs + ORC_EPS * h * h);
        av = -visco * c0 * mu / rho0;
    }
    return av;
}

/* Density_Diffusion_term_FOURTAKAS, src/SPH_viscouse_forces.h:45-61 */
static inline double fourtakas(double h, double drs, double dr_z, double drdW,
                               double arho, double nrho, double rho0,
                               double c0, double delta, double m,
                               double gravity) {
    const double cb = c0 * c0 * rho0 / 7.;
    const double dpH = 1. + dr_z * rho0 * gravity / cb;
    const double drhoH = rho0 * pow(dpH, 1. / 7) - rho0;
    const double psi =
        2. * c0 * h * delta * ((nrho - arho) - drhoH) / (drs * drs + ORC_EPS * h * h);
    return psi * drdW * m / nrho;
}

/* --------------------------------------------------------- neighbour grid */

/* Divide_To_Cells, src/SPH_find_pairs.h:5-42 */
void orc_divide_to_cells(orc_sys *s) {
    const double kh = s->kap * s->h;
    const double of = s->h * 0.273;
    s->ncx = (int)((s->xm - s->x0 + of) / kh) + 1;
    s->ncy = (int)((s->ym - s->y0 + of) / kh) + 1;
    s->ncells = s->ncx * s->ncy;
    s->cell_start = orc_xrealloc(s->cell_start, sizeof(int) * (s->ncells + 1));
    s->cell_count = orc_xrealloc(s->cell_count, sizeof(int) * (s->ncells + 1));
    memset(s->cell_start, 0, sizeof(int) * (s->ncells + 1));
    s->cells_built = 0;
}

/* Clear_cells, src/SPH_find_pairs.h:74-92 */
void orc_clear_cells(orc_sys *s) {
    if (s->cell_start) memset(s->cell_start, 0, sizeof(int) * (s->ncells + 1));
    s->cells_built = 0;
}

/* cell of a point: src/SPH_find_pairs.h:64-65 (POS, src/SPH_defs.h:36).
 * Returns -1 when the point lies outside the grid. */
static inline int cell_of(const orc_sys *s, double x, double y) {
    const double kh = s->kap * s->h;
    const double of = s->h * 0.273;
    const int npx = (int)((x - s->x0 + of) / kh);
    const int npy = (int)((y - s->y0 + of) / kh);
    if (npx < 0 || npy < 0 || npx >= s->ncx || npy >= s->ncy) return -1;
    return npy + npx * s->ncy;
}

/* Particle_To_Cell, src/SPH_find_pairs.h:45-72.  The reference appends
 * particles serially in index order, so each cell list is ascending; the
 * CSR build below visits particles in the same order. */
void orc_particle_to_cell(orc_sys *s) {
    const int nc = s->ncells;
    int *cnt = s->cell_count;
    memset(cnt, 0, sizeof(int) * (nc + 1));
    s->cell_list = orc_xrealloc(s->cell_list, sizeof(int) * (s->np ? s->np : 1));
    int *key = malloc(sizeof(int) * (s->np ? s->np : 1));
    if (!key) abort();
    s->escaped = 0;
    for (int p = 0; p < s->np; p++) {
        key[p] = cell_of(s, s->rx[p], s->ry[p]);
        if (key[p] < 0) {
            s->escaped++;
            continue;
        }
        cnt[key[p]]++;
    }
    int acc = 0;
    for (int c = 0; c < nc; c++) {
        s->cell_start[c] = acc;
        acc += cnt[c];
        cnt[c] = s->cell_start[c];
    }
    s->cell_start[nc] = acc;
    for (int p = 0; p < s->np; p++)
        if (key[p] >= 0) s->cell_list[cnt[key[p]]++] = p;
    free(key);
    s->cells_built = 1;
}

/* ------------------------------------------------------------ pressure */

/* Density_to_pressure, src/SPH_pressure.h:65-89 (the rho range warning is a
 * print in the reference and has no effect on the state). */
void orc_density_to_pressure(orc_sys *s) {
#pragma omp parallel for schedule(static)
    for (int p = 0; p < s->np; p++)
        s->p[p] = orc_pressure(s->rho[p], s->rho0, s->cs);
}

/* ---------------------------------------------------------- pair loop */

/* Compute_Forces, mDBC flavour src/SPH_interaction.h:8-149 and DBC flavour
 * src/SPH_interactionDBC.h:8-155.  Cell-parallel; each row is written by the
 * one thread that owns its cell, and the summation order per row is the
 * reference's (neighbour cells zz,zp,pp,pz,pm,zm,mm,mz,mp, each list
 * ascending), so the result does not depend on the thread count. */
/* Compute_Forces of the boundary-integral flavour, src/SPH_interactionBT.h:
 * fluid rows only; a fluid neighbour contributes as in SPH_interaction.h, a
 * wall neighbour b with normal n_b contributes W (p_temp + visco) dp n_b rho_b
 * to the momentum sum and -(dv . n_b) W rho_b dp to the continuity sum (no
 * diffusion term); both sums are divided by the Shepard sum gamma =
 * sum over fluid neighbours of W m / rho_b when gamma > eps, else a = -g and
 * drho = 0 (:52-187). */
static void bt_forces(orc_sys *s) {
    const int ncy = s->ncy;
    const int nc = s->ncells;
    const double h = s->h, m = s->m, c0 = s->cs, delta = s->delta, dp = s->dp;
    const double rho0 = s->rho0, gy = s->gravy, alpha = s->avisc;
    const int *cs = s->cell_start, *cl = s->cell_list;

#pragma omp parallel for schedule(dynamic, 3)
    for (int c = 0; c < nc; c++) {
        const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                           c + ncy,     c - 1 + ncy, c - 1,
                           c - 1 - ncy, c - ncy,     c + 1 - ncy};
        for (int i = cs[c]; i < cs[c + 1]; i++) {
            const int ai = cl[i];
            if (s->type[ai] != ORC_FLUID) continue;
            const double arx = s->rx[ai], ary = s->ry[ai];
            const double avx = s->vx[ai], avy = s->vy[ai];
            const double arho = s->rho[ai], ap = s->p[ai];
            double acx = 0., acy = 0., drho_sum = 0., diff_sum = 0., gamma = 0.;
            for (int k = 0; k < 9; k++) {
                const int cc = ac[k];
                if (cc < 0 || cc >= nc) continue;
                for (int n = cs[cc]; n < cs[cc + 1]; n++) {
                    const int ni = cl[n];
                    if (ai == ni) continue;
                    const double nrx = s->rx[ni], nry = s->ry[ni];
                    const double nvx = s->vx[ni], nvy = s->vy[ni];
                    const double nrho = s->rho[ni], npr = s->p[ni];
                    const double drx = arx - nrx, dry = ary - nry;
                    const double dvx = avx - nvx, dvy = avy - nvy;
                    const double drs = sqrt((drx * drx) + (dry * dry));
                    const double drdv = drx * dvx + dry * dvy;
                    double W, F;
                    orc_wendland(drs, h, &W, &F);
                    const double dWx = drx * F, dWy = dry * F;
                    const double dvdW = dvx * dWx + dvy * dWy;
                    const double drdW = drx * dWx + dry * dWy;
                    const double p_temp = (ap + npr) / (arho * nrho);
                    const double visco =
                        av_term(h, drs, drdv, 0.5 * (arho + nrho), c0, alpha);
                    const int wall = s->type[ni] == ORC_WALL;
                    if (wall) {
                        const double nbx = ni < s->nn ? s->nx[ni] : 0.;
                        const double nby = ni < s->nn ? s->ny[ni] : 0.;
                        acx += W * (p_temp + visco) * dp * nbx * nrho;
                        acy += W * (p_temp + visco) * dp * nby * nrho;
                        const double dvnb = dvx * nbx + dvy * nby;
                        drho_sum -= dvnb * W * nrho * dp;
                    } else {
                        acx -= dWx * (p_temp + visco) * m;
                        acy -= dWy * (p_temp + visco) * m;
                        const double dt_ = fourtakas(h, drs, dry, drdW, arho, nrho,
                                                     rho0, c0, delta, m, gy);
                        drho_sum += dvdW * m;
                        diff_sum -= dt_;
                    }
                    if (s->type[ni] == ORC_FLUID) gamma += W * m / nrho;
                }
            }
            if (gamma > ORC_EPS) {
                s->ax[ai] = acx / gamma - 0.;
                s->ay[ai] = acy / gamma - gy;
                s->drho[ai] = drho_sum / gamma + diff_sum / gamma;
            } else {
                s->ax[ai] = 0. - 0.;
                s->ay[ai] = 0. - gy;
                s->drho[ai] = 0;
            }
        }
    }
}

/* BT_compute_density_BTGeo, src/SPH_BT.h:9-50, with
 * Kernel_density_approximation_BT_update, src/SPH_kernel_approx.h:1838-1953:
 * each wall particle gets the Shepard density of the fluid around its own
 * position, sum m W / sum m W / rho over the 3x3 cell block (1000 when the
 * sum is 0), raised to at least 1000. */
void orc_bt_density(orc_sys *s) {
    const double kh = s->kap * s->h, of = s->h * 0.273, h = s->h, m = s->m;
    const int ncy = s->ncy, nc = s->ncells;
    const int *cs = s->cell_start, *cl = s->cell_list;
#pragma omp parallel for schedule(static)
    for (int p = 0; p < s->np; p++) {
        if (s->type[p] != ORC_WALL) continue;
        const double arx = s->rx[p], ary = s->ry[p];
        const int npx = (int)((arx - s->x0 + of) / kh);
        const int npy = (int)((ary - s->y0 + of) / kh);
        const int c = npy + npx * ncy;
        const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                           c + ncy,     c - 1 + ncy, c - 1,
                           c - 1 - ncy, c - ncy,     c + 1 - ncy};
        double Wsum = 0., rhoWsum = 0.;
        for (int k = 0; k < 9; k++) {
            const int cc = ac[k];
            if (cc < 0 || cc >= nc) continue;
            for (int n = cs[cc]; n < cs[cc + 1]; n++) {
                const int ni = cl[n];
                if (s->type[ni] != ORC_FLUID) continue;
                const double drx = arx - s->rx[ni], dry = ary - s->ry[ni];
                const double drs = sqrt(drx * drx + dry * dry);
                double W, F;
                orc_wendland(drs, h, &W, &F);
                Wsum += W * m / s->rho[ni];
                rhoWsum += m * W;
            }
        }
        double dens = Wsum > 0. ? rhoWsum / Wsum : 1000.;
        if (dens < 1000.) dens = 1000.;
        s->rho[p] = dens;
    }
}

void orc_compute_forces(orc_sys *s, int model) {
    if (model == ORC_BT) {
        bt_forces(s);
        return;
    }
    const int ncy = s->ncy;
    const int nc = s->ncells;
    const double h = s->h, m = s->m, c0 = s->cs, delta = s->delta;
    const double rho0 = s->rho0, gy = s->gravy, alpha = s->avisc;
    const int *cs = s->cell_start, *cl = s->cell_list;

#pragma omp parallel for schedule(dynamic, 3)
    for (int c = 0; c < nc; c++) {
        const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                           c + ncy,     c - 1 + ncy, c - 1,
                           c - 1 - ncy, c - ncy,     c + 1 - ncy};
        for (int i = cs[c]; i < cs[c + 1]; i++) {
            const int ai = cl[i];
            const int at = s->type[ai];
            if (model == ORC_MDBC) {
                if (at != ORC_FLUID) continue;
            }
            const double arx = s->rx[ai], ary = s->ry[ai];
            const double avx = s->vx[ai], avy = s->vy[ai];
            const double arho = s->rho[ai], ap = s->p[ai];
            double acx = 0., acy = 0., drho_sum = 0., diff_sum = 0.;
            for (int k = 0; k < 9; k++) {
                const int cc = ac[k];
                if (cc < 0 || cc >= nc) continue;
                for (int n = cs[cc]; n < cs[cc + 1]; n++) {
                    const int ni = cl[n];
                    if (ai == ni) continue;
                    if (model == ORC_DBC && at == ORC_WALL && s->type[ni] == ORC_WALL)
                        continue;
                    const double nrx = s->rx[ni], nry = s->ry[ni];
                    const double nvx = s->vx[ni], nvy = s->vy[ni];
                    const double nrho = s->rho[ni], npr = s->p[ni];
                    const double drx = arx - nrx, dry = ary - nry;
                    const double dvx = avx - nvx, dvy = avy - nvy;
                    const double drs = sqrt((drx * drx) + (dry * dry));
                    const double drdv = drx * dvx + dry * dvy;
                    double W, F;
                    orc_wendland(drs, h, &W, &F);
                    const double dWx = drx * F, dWy = dry * F;
                    const double dvdW = dvx * dWx + dvy * dWy;
                    const double drdW = drx * dWx + dry * dWy;
                    const double p_temp = (ap + npr) / (arho * nrho);
                    const double visco =
                        av_term(h, drs, drdv, 0.5 * (arho + nrho), c0, alpha);
                    acx -= dWx * (p_temp + visco) * m;
                    acy -= dWy * (p_temp + visco) * m;
                    const double dt_ = fourtakas(h, drs, dry, drdW, arho, nrho,
                                                 rho0, c0, delta, m, gy);
                    drho_sum += dvdW * m;
                    diff_sum -= dt_;
                }
            }
            if (model == ORC_DBC && at == ORC_WALL) {
                s->ax[ai] = 0.;
                s->ay[ai] = 0.;
            } else {
                s->ax[ai] = acx - 0.;
                s->ay[ai] = acy - gy;
            }
            s->drho[ai] = drho_sum + diff_sum;
        }
    }
}

/* ---------------------------------------------------------------- mDBC */

/* determinant, src/SPH_kernel_approx.h:663-675 */
static inline double det3(double a11, double a12, double a13, double a21,
                          double a22, double a23, double a31, double a32,
                          double a33) {
    return (a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 -
            a31 * a22 * a13 - a32 * a23 * a11 - a33 * a21 * a12);
}

/* Kernel_density_approximation_MATRIX_mDBC, src/SPH_kernel_approx.h:1141-1343:
 * first-order corrected density at the ghost node (gx, gy), extrapolated by
 * gnd = r_wall - r_ghost. */
static double mdbc_ghost_density(const orc_sys *s, double gx, double gy,
                                 double gndx, double gndy) {
    const double kh = s->kap * s->h;
    const double of = s->h * 0.273;
    const double h = s->h, m = s->m;
    const int ncy = s->ncy, nc = s->ncells;
    const int npx = (int)((gx - s->x0 + of) / kh);
    const int npy = (int)((gy - s->y0 + of) / kh);
    const int c = npy + npx * ncy;
    const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                       c + ncy,     c - 1 + ncy, c - 1,
                       c - 1 - ncy, c - ncy,     c + 1 - ncy};
    double a11 = 0, a12 = 0, a13 = 0, a21 = 0, a22 = 0, a23 = 0, a31 = 0,
           a32 = 0, a33 = 0;
    double drhodx = 0, drhody = 0, rhoWsum = 0;
    for (int k = 0; k < 9; k++) {
        const int cc = ac[k];
        if (cc < 0 || cc >= nc) continue;
        for (int n = s->cell_start[cc]; n < s->cell_start[cc + 1]; n++) {
            const int ni = s->cell_list[n];
            if (s->type[ni] != ORC_FLUID) continue;
            const double nrho = s->rho[ni];
            const double drx = gx - s->rx[ni], dry = gy - s->ry[ni];
            const double drs = sqrt(drx * drx + dry * dry);
            double W, F;
            orc_wendland(drs, h, &W, &F);
            rhoWsum += m * W;
            drhodx += drx * F * m;
            drhody += dry * F * m;
            a11 += W * (m / nrho);
            a12 += drx * W * (m / nrho);
            a13 += dry * W * (m / nrho);
            a21 += drx * F * (m / nrho);
            a22 += drx * drx * F * (m / nrho);
            a23 += drx * dry * F * (m / nrho);
            a31 += dry * F * (m / nrho);
            a32 += dry * drx * F * (m / nrho);
            a33 += dry * dry * F * (m / nrho);
        }
    }
    const double det = det3(a11, a12, a13, a21, a22, a23, a31, a32, a33);
    double dens;
    if (det > 0.001) {
        const double i11 = (a22 * a33 - a23 * a32) / det;
        const double i12 = -(a12 * a33 - a13 * a32) / det;
        const double i13 = (a12 * a23 - a13 * a22) / det;
        const double i21 = -(a21 * a33 - a23 * a31) / det;
        const double i22 = (a11 * a33 - a13 * a31) / det;
        const double i23 = -(a11 * a23 - a13 * a21) / det;
        const double i31 = (a21 * a32 - a22 * a31) / det;
        const double i32 = -(a11 * a32 - a12 * a31) / det;
        const double i33 = (a11 * a22 - a12 * a21) / det;
        const double dens_temp = rhoWsum * i11 + drhodx * i12 + drhody * i13;
        const double grx = -(rhoWsum * i21 + drhodx * i22 + drhody * i23);
        const double gry = -(rhoWsum * i31 + drhodx * i32 + drhody * i33);
        dens = (dens_temp + grx * gndx + gry * gndy);
    } else if (a11 > 0) {
        dens = rhoWsum / a11;
    } else {
        dens = 1000.;
    }
    return dens;
}

/* mDBC_compute_density_mdbcGeo, src/SPH_mDBC.h:9-50 */
void orc_mdbc_density(orc_sys *s) {
#pragma omp parallel for schedule(static)
    for (int p = 0; p < s->np; p++) {
        if (s->type[p] != ORC_WALL) continue;
        if (p >= s->ngnr) continue; /* the reference would read past gnr */
        const double rx = s->rx[p], ry = s->ry[p];
        const double gx = s->gx[p], gy = s->gy[p];
        const double gndx = rx - gx, gndy = ry - gy;
        double r = mdbc_ghost_density(s, gx, gy, gndx, gndy);
        if (r < 1000.) r = 1000.;
        s->rho[p] = r;
    }
}

/* ---------------------------------------------------------- integration */

/* Integrate_SymplecticPredictor, src/SPH_integration.h:266-287 */
void orc_predictor(orc_sys *s, double dt) {
#pragma omp parallel for schedule(static)
    for (int p = 0; p < s->np; p++) {
        s->rho_o[p] = s->rho[p];
        s->rox[p] = s->rx[p];
        s->roy[p] = s->ry[p];
        s->vox[p] = s->vx[p];
        s->voy[p] = s->vy[p];
        s->rho[p] = s->rho[p] + s->drho[p] * dt * 0.5;
        s->rx[p] = s->rx[p] + s->vx[p] * dt * 0.5;
        s->ry[p] = s->ry[p] + s->vy[p] * dt * 0.5;
        s->vx[p] = s->vx[p] + s->ax[p] * dt * 0.5;
        s->vy[p] = s->vy[p] + s->ay[p] * dt * 0.5;
    }
    s->cells_built = 0;
}

/* Integrate_SymplecticCorrector, src/SPH_integration.h:289-309 */
void orc_corrector(orc_sys *s, double dt) {
#pragma omp parallel for schedule(static)
    for (int p = 0; p < s->np; p++) {
        const double epsilon = (-s->drho[p] / s->rho[p]) * dt;
        s->rho[p] = s->rho_o[p] * ((2. - epsilon) / (2. + epsilon));
        s->vx[p] = s->vox[p] + s->ax[p] * dt;
        s->vy[p] = s->voy[p] + s->ay[p] * dt;
        s->rx[p] = s->rox[p] + (s->vx[p] + s->vox[p]) * dt * 0.5;
        s->ry[p] = s->roy[p] + (s->vy[p] + s->voy[p]) * dt * 0.5;
    }
    s->cells_built = 0;
}

/* Remove_particle, src/SPH_particle_system.h:110-146 (order-preserving
 * erase of every per-particle vector; gnr is not touched, :144) */
void orc_erase_particle(orc_sys *s, int p) {
    const int tail = s->np - p - 1;
#define E(f) memmove(s->f + p, s->f + p + 1, sizeof(s->f[0]) * tail)
    E(index); E(type); E(p); E(rho); E(drho); E(rx); E(ry); E(vx); E(vy);
    E(ax); E(ay); E(rox); E(roy); E(vox); E(voy); E(rho_o);
    if (s->ale) {
        E(om); E(omr); E(omvx); E(omvy); E(om_o); E(omr_o); E(omvx_o); E(omvy_o);
        E(dom); E(domr); E(domvx); E(domvy);
        for (int k = 0; k < 12; k++) E(grad[k]);
        if (p < s->nn) {
            memmove(s->nx + p, s->nx + p + 1, sizeof(double) * (s->nn - p - 1));
            memmove(s->ny + p, s->ny + p + 1, sizeof(double) * (s->nn - p - 1));
            s->nn--;
        }
    }
#undef E
    s->np--;
}

/* RemoveParticlesOutOfDomain, src/SPH_btdebug.h:4-31.  The reference erases
 * inside a forward loop without stepping back, so the particle that slides
 * into slot p is not examined in that call; the same happens here. */
int orc_remove_out_of_domain(orc_sys *s) {
    const double x0 = s->x0, xm = s->xm, y0 = s->y0, ym = s->ym;
    int removed = 0;
    for (int p = 0; p < s->np; p++) {
        if (s->type[p] != ORC_FLUID) continue;
        const double rx = s->rx[p], ry = s->ry[p];
        if ((ry < (y0 - ORC_EPS)) || (ry > ym + ORC_EPS) || (rx < x0 - ORC_EPS) ||
            (rx > xm - ORC_EPS)) {
            orc_erase_particle(s, p);
            removed++;
        }
    }
    if (removed) s->cells_built = 0;
    return removed;
}

/* One RUN-loop body: cases/damBreakLong_mDBC/SPH_simulationSymplectic.h:54-118
 * (mDBC) and cases/stillWater_DBC/SPH_simulationSymplectic.h:53-118 (DBC; the
 * mDBC call is commented out there).  Output/probe blocks are not part of the
 * step. */
void orc_step(orc_sys *s, int model, double dt, int nsteps) {
    for (int k = 0; k < nsteps; k++) {
        if (model == ORC_MDBC) {
            orc_mdbc_density(s);
            orc_density_to_pressure(s);
        } else if (model == ORC_BT) {  /* cases/damBreakLong_BT/SPH_simulationSymplectic.h */
            orc_bt_density(s);
            orc_density_to_pressure(s);
        }
        orc_predictor(s, dt);
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

/* Pair-set digest over the reference's 3x3 cell block of every particle
 * (src/SPH_interaction.h:26-36, neighbour loop :71-82): for each row, the
 * count, sum and xor of the original indices of neighbours j != i with
 * r/h <= 2 (the support of the Wendland kernel, src/SPH_kernel.h:63).  Fluid
 * rows see every neighbour; wall rows see fluid only (the DBC flavour skips
 * wall-wall pairs, src/SPH_interactionDBC.h:84).  Outputs in particle order. */
void orc_pair_digest(const orc_sys *s, int *count, long long *sum, int *xr) {
    const int ncy = s->ncy, nc = s->ncells;
    const int *cs = s->cell_start, *cl = s->cell_list;
#pragma omp parallel for schedule(dynamic, 64)
    for (int c = 0; c < nc; c++) {
        const int ac[9] = {c,           c + 1,       c + 1 + ncy,
                           c + ncy,     c - 1 + ncy, c - 1,
                           c - 1 - ncy, c - ncy,     c + 1 - ncy};
        for (int i = cs[c]; i < cs[c + 1]; i++) {
            const int ai = cl[i];
            int cnt = 0, x = 0;
            long long sm = 0;
            for (int k = 0; k < 9; k++) {
                const int cc = ac[k];
                if (cc < 0 || cc >= nc) continue;
                for (int n = cs[cc]; n < cs[cc + 1]; n++) {
                    const int ni = cl[n];
                    if (ni == ai) continue;
                    if (s->type[ai] == ORC_WALL && s->type[ni] == ORC_WALL) continue;
                    const double drx = s->rx[ai] - s->rx[ni], dry = s->ry[ai] - s->ry[ni];
                    const double drs = sqrt((drx * drx) + (dry * dry));
                    if (drs / s->h <= 2.0) {
                        cnt++;
                        sm += s->index[ni];
                        x ^= s->index[ni];
                    }
                }
            }
            count[ai] = cnt;
            sum[ai] = sm;
            xr[ai] = x;
        }
    }
}
