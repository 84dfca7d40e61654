/*
 * tsph_oracle_internal.h -- the oracle's state (TEST INFRASTRUCTURE), shared
 * by oracle/tsph_oracle.c (WCSPH) and oracle/tsph_oracle_ale.c (ALE-SPH).
 */
#ifndef TSPH_ORACLE_INTERNAL_H
#define TSPH_ORACLE_INTERNAL_H

#include <stddef.h>

#define ORC_EPS 0.01 /* src/SPH_defs.h:69 */

/* BufferZone, src/SPH_inlet_outlet_data.h (inlet / outlet buffer zones) */
typedef struct {
    double ox, oy;          /* orientation {+-1, 0} or {0, +-1} */
    double x0, y0, xm, ym;  /* zone region */
    int nbl;                /* buffer layers */
    double bl, bh;          /* buffer length, height */
    int btype;              /* particle type of the zone's buffer particles */
    double vbx, vby;        /* buffer velocity */
} orc_zone;

#define ORC_MAX_ZONES 8

struct orc_sys {
    int np, cap;
    int *index;
    int *type;
    double *p, *rho, *drho;
    double *rx, *ry, *vx, *vy, *ax, *ay;
    double *rox, *roy, *vox, *voy, *rho_o;
    /* mDBC ghost nodes, indexed by particle index (src/SPH_data.h:51) */
    int ngnr, gcap;
    double *gx, *gy;
    /* SPH_constants (src/SPH_data.h:30-46) */
    double h, kap, dp, cs, rho0, gravy, avisc, delta, m;
    /* Simulation_data (src/SPH_data.h:111-122): padded domain */
    double x0, xm, y0, ym;
    /* cells as CSR: cell c holds cell_list[cell_start[c] .. cell_start[c+1]) */
    int ncx, ncy, ncells;
    int *cell_start, *cell_list, *cell_count;
    int cells_built;
    int escaped;
    /* ALE-SPH fields (special.*, src/SPH_data.h:54-79): omega, omega*rho,
     * omega*v, their copies of the leap-frog, their rates, the MUSCL
     * gradients (rho, vx, vy forward then backward, x and y each) and the
     * boundary normals of BT walls (special.n, indexed by particle index) */
    int ale;
    int ale_scheme; /* 0: fluxes as the reference writes them; 1: MUSCL states */
    double *om, *omr, *omvx, *omvy, *om_o, *omr_o, *omvx_o, *omvy_o;
    double *dom, *domr, *domvx, *domvy;
    double *grad[12];
    int nn, ncap;
    double *nx, *ny;
    /* open boundaries (particles.zones, src/SPH_particle_system.h:21) */
    int nzones;
    orc_zone zones[ORC_MAX_ZONES];
};


void *orc_xrealloc(void *p, size_t n);
void orc_grow(orc_sys *s, int need);
void orc_erase_particle(orc_sys *s, int p);
void orc_wendland(double r, double h, double *w, double *f);
double orc_pressure(double rho, double rho0, double c0);

#endif
