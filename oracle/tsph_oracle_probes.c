/*
 * tsph_oracle_probes.c -- CPU oracle of the case drivers' probes
 * (TEST INFRASTRUCTURE): the water level of src/SPH_water_level.h:6-150 and
 * the Shepard point interpolation behind Pressure_in_point
 * (src/SPH_measure_pressure.h:6-15, src/testing.h:6-149), in FP64 and in the
 * reference's operation order.  Pinned bit-for-bit against the reference
 * compiled from its own headers (oracle/ref_harness.cpp).
 */
#include <math.h>

#include "tsph_oracle.h"
#include "tsph_oracle_internal.h"

/* cell of a point and its 3 x 3 block in the reference's order
 * (zz, zp, pp, pz, pm, zm, mm, mz, mp); blocks below 0 are skipped as in the
 * reference, blocks at or above ncells too (the reference would read past
 * its cell array there) */
static void probe_cells(const orc_sys *s, double x, double y, int ac[9]) {
    const double kh = s->kap * s->h, of = s->h * 0.273;
    const unsigned int npx = (unsigned int)(int)((x - s->x0 + of) / kh);
    const unsigned int npy = (unsigned int)(int)((y - s->y0 + of) / kh);
    const int ncy = s->ncy;
    const int c = (int)(npy + npx * (unsigned int)ncy);
    const int a[9] = {c,           c + 1,       c + 1 + ncy,
                      c + ncy,     c - 1 + ncy, c - 1,
                      c - 1 - ncy, c - ncy,     c + 1 - ncy};
    for (int k = 0; k < 9; k++) ac[k] = (a[k] < 0 || a[k] >= s->ncells) ? -1 : a[k];
}

/* Sum_kernel_function, src/SPH_water_level.h:6-80: sum of m W / rho over
 * every particle (fluid and walls) of the block */
static double kernel_volume(const orc_sys *s, double x, double y) {
    int ac[9];
    probe_cells(s, x, y, ac);
    double mWsum = 0;
    for (int k = 0; k < 9; k++) {
        const int cl = ac[k];
        if (cl < 0) continue;
        for (int n = s->cell_start[cl]; n < s->cell_start[cl + 1]; n++) {
            const int p = s->cell_list[n];
            const double dx = x - s->rx[p], dy = y - s->ry[p];
            const double drs = sqrt(pow(dx, 2) + pow(dy, 2));
            double W, F;
            orc_wendland(drs, s->h, &W, &F);
            mWsum += s->m * W / s->rho[p];
        }
    }
    return mWsum;
}

/* Water_Elevation / Water_Elevation_inverse, src/SPH_water_level.h:84-150:
 * samples upwards (downwards) from y0 with the growing step i * dp_wl until
 * the kernel volume drops to (reaches) 0.5; NaN if it never does */
double orc_water_level(orc_sys *s, double x, double y0, int inverse) {
    const double dp_wl = s->dp * 0.00005;
    double ay = y0;
    const int nmax = (int)(s->ym / dp_wl);
    for (int i = 0; i < nmax; i++) {
        if (inverse) {
            ay -= i * dp_wl;
            if (kernel_volume(s, x, ay) >= 0.5) return ay + i * dp_wl;
        } else {
            ay += i * dp_wl;
            if (kernel_volume(s, x, ay) <= 0.5) return ay - i * dp_wl;
        }
    }
    return NAN;
}

/* Kernel_velocity_approximation_TEST, src/testing.h:6-149: Shepard averages
 * {rho, p, vx, vy} at a point where the kernel volume exceeds 0.5, else 0 */
void orc_point_fields(orc_sys *s, double x, double y, double out[4]) {
    int ac[9];
    probe_cells(s, x, y, ac);
    double Wsum = 0, vWx = 0, vWy = 0, rhoW = 0, pW = 0, mWsum = 0;
    for (int k = 0; k < 9; k++) {
        const int cl = ac[k];
        if (cl < 0) continue;
        for (int n = s->cell_start[cl]; n < s->cell_start[cl + 1]; n++) {
            const int q = s->cell_list[n];
            const double dx = x - s->rx[q], dy = y - s->ry[q];
            const double drs = sqrt(pow(dx, 2) + pow(dy, 2));
            double W, F;
            orc_wendland(drs, s->h, &W, &F);
            Wsum += W;
            vWx = vWx + s->vx[q] * W;
            vWy = vWy + s->vy[q] * W;
            rhoW = rhoW + s->rho[q] * W;
            pW = pW + s->p[q] * W;
            mWsum += s->m * W / s->rho[q];
        }
    }
    double vx = 0., vy = 0., rho = 0., p = 0.;
    if (mWsum > 0.5) {
        vx = vx + vWx / Wsum;
        vy = vy + vWy / Wsum;
        rho = rho + rhoW / Wsum;
        p = p + pW / Wsum;
    }
    if (Wsum == 0) {
        vx = 0.;
        vy = 0.;
    }
    out[0] = rho;
    out[1] = p;
    out[2] = vx;
    out[3] = vy;
}
