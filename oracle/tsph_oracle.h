/*
 * tsph_oracle.h -- CPU oracle for the 2D WCSPH time step (TEST INFRASTRUCTURE).
 *
 * This is the checker, not the product: only the tests, the smoke check and
 * the CPU-baseline leg of bench.py may load it.  It restates, in plain C and
 * IEEE double precision, the reference (tomashalada/tinySPH_old, header-only
 * C++) functions on the time-step path, in the same floating-point operation
 * order, so that with one thread its results are bit-identical to the
 * reference compiled from its own sources (see oracle/ref_harness.cpp and
 * tests/golden/).  Each function cites the reference file:line it follows.
 *
 * State is kept in the reference's own particle order (array index = the
 * reference's particle index, erase-preserving), as structure-of-arrays.
 */
#ifndef TSPH_ORACLE_H
#define TSPH_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sys orc_sys;

/* wall models of Compute_Forces */
#define ORC_MDBC 0   /* src/SPH_interaction.h     */
#define ORC_DBC 1    /* src/SPH_interactionDBC.h  */
#define ORC_BT 2     /* src/SPH_interactionBT.h: boundary-integral walls with normals
                        (added with orc_ale_add_normal, walls first) */

/* particle types, src/SPH_defs.h:44-48 */
#define ORC_FLUID 0
#define ORC_WALL 1

/* state field ids for orc_get_field / orc_set_field */
enum {
    ORC_F_RX = 0, ORC_F_RY, ORC_F_VX, ORC_F_VY, ORC_F_AX, ORC_F_AY,
    ORC_F_RHO, ORC_F_DRHO, ORC_F_P,
    ORC_F_ROX, ORC_F_ROY, ORC_F_VOX, ORC_F_VOY, ORC_F_RHO_O,
    ORC_F_NFIELDS
};

orc_sys *orc_create(double h, double kap, double cs, double rho0, double visco,
                    double delta, double dp, double x0, double xm, double y0,
                    double ym);
void orc_destroy(orc_sys *s);
void orc_set_threads(int n);
int orc_get_threads(void);

void orc_add_particle(orc_sys *s, int type, double p, double rho, double rx,
                      double ry, double vx, double vy, double ax, double ay);
void orc_add_gnr(orc_sys *s, double gx, double gy);

int orc_np(const orc_sys *s);
void orc_grid(const orc_sys *s, int *ncx, int *ncy);
double orc_const(const orc_sys *s, int which); /* 0 h,1 kap,2 dp,3 cs,4 rho0,5 avisc,6 delta,7 m,8 g */

void orc_get_field(const orc_sys *s, int field, double *out);
void orc_set_field(orc_sys *s, int field, const double *in);
void orc_get_meta(const orc_sys *s, int *index, int *type);
int orc_get_cells(const orc_sys *s, int *cell_start, int *cell_list);

/* the reference entry points */
void orc_divide_to_cells(orc_sys *s);
void orc_clear_cells(orc_sys *s);
void orc_particle_to_cell(orc_sys *s);
void orc_density_to_pressure(orc_sys *s);
void orc_compute_forces(orc_sys *s, int model);
void orc_mdbc_density(orc_sys *s);
/* open boundaries: BufferZone(x0, xm, y0, ym, nbl, v0, orientation, btype)
 * (src/SPH_inlet_outlet_data.h) appended to particles.zones; returns its
 * index or -1 */
int orc_add_zone(orc_sys *s, double x0, double xm, double y0, double ym, int nbl, double vx,
                 double vy, double ox, double oy, int btype);
/* BZ_Integrate_inlet / BZ_Integrate_outlet, src/SPH_buffer_zones.h:10-206 */
void orc_bz_inlet(orc_sys *s, int zone, double dt);
void orc_bz_outlet(orc_sys *s, int zone, double dt);
/* RUN of cases/inflowSlab_mDBC and cases/flowDrop_mDBC
 * SPH_simulationSymplectic.h: the mDBC step with every zone's
 * BZ_Integrate_inlet (types 6-10) or BZ_Integrate_outlet (11-15), in zone
 * order, after the predictor */
void orc_step_zones(orc_sys *s, int model, double dt, int nsteps);
void orc_bt_density(orc_sys *s);
void orc_predictor(orc_sys *s, double dt);
void orc_corrector(orc_sys *s, double dt);
int orc_remove_out_of_domain(orc_sys *s);
/* one RUN-loop body per step (mDBC or DBC case driver order) */
void orc_step(orc_sys *s, int model, double dt, int nsteps);

/* in-support pair-set digest (count, sum and xor of neighbour indices) */
void orc_pair_digest(const orc_sys *s, int *count, long long *sum, int *xr);

/* ---- ALE-SPH (cases/ALESPH_dambreakLong/MUSCL.h path) ---- */
/* probes of the case drivers: water level (src/SPH_water_level.h:84-150) and
 * Shepard point fields {rho, p, vx, vy} (src/testing.h:6-149) */
double orc_water_level(orc_sys *s, double x, double y0, int inverse);
void orc_point_fields(orc_sys *s, double x, double y, double out[4]);

void orc_ale_add_particle(orc_sys *s, int type, double p, double rho, double rx, double ry,
                          double vx, double vy);
void orc_ale_add_normal(orc_sys *s, double nx, double ny);
void orc_ale_get_field(const orc_sys *s, int f, double *out);
void orc_ale_set_field(orc_sys *s, int f, const double *in);
/* 0: the reference's MUSCL.h fluxes (default); 1: superbee MUSCL interface
 * states of both particles (no counterpart in the reference); 2: the
 * first-order fluxes of SPH_simulationINT.h (src/RALESPH_interaction.h) */
void orc_ale_set_scheme(orc_sys *s, int scheme);
void orc_ale_gradient(orc_sys *s);
void orc_ale_forces(orc_sys *s, double dt);
/* the first-order variant, src/RALESPH_interaction.h:12-289 (scheme 2 in
 * orc_ale_step) */
void orc_ale_forces_first_order(orc_sys *s);
void orc_ale_leapfrog_one(orc_sys *s, double dt);
void orc_ale_leapfrog_two(orc_sys *s, double dt, int step);
void orc_ale_step(orc_sys *s, double dt, int step0, int nsteps);

/* scalar kernels, exported for unit tests */
void orc_wendland(double r, double h, double *w, double *f);
double orc_pressure(double rho, double rho0, double c0);
double orc_pressure_to_density(double p, double rho0, double c0);

#ifdef __cplusplus
}
#endif
#endif
