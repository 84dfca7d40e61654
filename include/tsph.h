/*
 * tsph.h -- C ABI of the GB300 (sm_103a) 2D weakly-compressible SPH step.
 *
 * A drop-in for the time-step path of tomashalada/tinySPH_old: the particle
 * system, the cell-list pair search, the WCSPH continuity/momentum pair loop
 * with delta-SPH (Fourtakas) diffusion and artificial viscosity, the DBC and
 * mDBC wall models and the symplectic integrator.  Every entry point below
 * names the reference function it replaces (file:line within the reference
 * project).  Plain C types only; the library owns its device memory.
 *
 * Conventions
 *  - Every call returns an int status: TSPH_OK (0) or a TSPH_ERR_* code.
 *    tsph_last_error() gives a message for the calling thread.
 *  - Host arrays are in the reference's particle order: ascending particle
 *    index among live particles (the reference erases removed particles
 *    without reordering, src/SPH_particle_system.h:110-146).  Vectors are
 *    interleaved (x0, y0, x1, y1, ...), doubles, like std::vector<tdouble2>.
 *  - One CUDA stream per system; calls on one handle are not thread-safe.
 *  - Walls are static: the reference's integrators move a wall particle by
 *    v*dt with v = 0 (its pair loops never give walls an acceleration), so
 *    wall particles are binned once and kept out of the per-step sort.
 */
#ifndef TSPH_H
#define TSPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TSPH_ABI_VERSION 1

/* ---- status codes ---- */
enum {
    TSPH_OK = 0,
    TSPH_ERR_ARG = 1,           /* bad argument (null, size, type, range)      */
    TSPH_ERR_CUDA = 2,          /* a CUDA runtime call failed                   */
    TSPH_ERR_STATE = 3,         /* call out of order (e.g. cells not built)     */
    TSPH_ERR_NOMEM = 4,         /* device or host allocation failed             */
    TSPH_ERR_NUMERIC = 5,       /* NaN/Inf found in the state                   */
    TSPH_ERR_DENSITY = 6,       /* density outside [0, 1500] (the reference's
                                   warning range, src/SPH_pressure.h:76-80)     */
    TSPH_ERR_ESCAPED = 7,       /* a particle left the cell grid                */
    TSPH_ERR_UNSUPPORTED = 8    /* feature outside this build's scope           */
};

/* health flags accumulated on the device (tsph_health) */
#define TSPH_HEALTH_NAN 0x1u
#define TSPH_HEALTH_DENSITY 0x2u
#define TSPH_HEALTH_ESCAPED 0x4u
#define TSPH_HEALTH_REMOVED 0x8u
/* a pipelined kernel gave up waiting for its own staging pipeline (a bounded
 * wait ran out; the step's results are not valid) */
#define TSPH_HEALTH_STALL 0x10u
/* a staged upload (tsph_upload_async) was not applied: some particle index is
 * no longer live (erased), so its rows do not map one to one onto the state */
#define TSPH_HEALTH_UPLOAD 0x20u

/* particle types, src/SPH_defs.h:44-48 (fluid = 0, wall = 1) */
enum { TSPH_FLUID = 0, TSPH_WALL = 1 };

/* wall models: Compute_Forces of src/SPH_interaction.h (mDBC: fluid rows only,
 * wall density from ghost nodes) and src/SPH_interactionDBC.h (DBC: walls get
 * a density rate from fluid neighbours) */
enum { TSPH_WALL_MDBC = 0, TSPH_WALL_DBC = 1, TSPH_WALL_BT = 2 };

/* arithmetic of the pair/integration kernels: FP32 pair math with FP64
 * positions (the production build), or FP64 throughout (the error study) */
enum { TSPH_PREC_FP32 = 0, TSPH_PREC_FP64 = 1 };

/* fields for tsph_download / tsph_upload (bit mask) */
enum {
    TSPH_F_R = 1 << 0,      /* double[2n] position            data.r    */
    TSPH_F_V = 1 << 1,      /* double[2n] velocity            data.v    */
    TSPH_F_A = 1 << 2,      /* double[2n] acceleration        data.a    */
    TSPH_F_RHO = 1 << 3,    /* double[n]  density             data.rho  */
    TSPH_F_DRHO = 1 << 4,   /* double[n]  density rate        data.drho */
    TSPH_F_P = 1 << 5,      /* double[n]  pressure            data.p    */
    TSPH_F_INDEX = 1 << 6,  /* int32[n]   original index      data.index     */
    TSPH_F_TYPE = 1 << 7    /* int32[n]   particle type       data.part_type */
};

/* SPH_constants, src/SPH_data.h:124-140; filled like the Particle_system
 * constructor (src/SPH_particle_system.h:191-212): gravity (0, 9.81) and
 * m = rho0 / (1/dp * 1/dp) are derived, not passed. */
typedef struct {
    double h;      /* smoothing length                       */
    double kap;    /* kernel support coefficient (kh = kap h) */
    double cs;     /* numerical speed of sound c0             */
    double rho0;   /* reference density                       */
    double visco;  /* artificial-viscosity alpha              */
    double delta;  /* delta-SPH coefficient                   */
    double dp;     /* initial particle spacing                */
} tsph_constants;

/* Simulation_data, src/SPH_data.h:205-219: the (padded) domain box */
typedef struct {
    double x_0, x_m, y_0, y_m;
} tsph_domain;

/* Host view of the particle state; any pointer may be NULL. */
typedef struct {
    double *r, *v, *a, *rho, *drho, *p;
    int32_t *index, *type;
} tsph_host_state;

typedef struct tsph_system tsph_system;

/* ---- library ---- */
int tsph_abi_version(void);
const char *tsph_last_error(void);
const char *tsph_status_string(int status);
/* number of visible CUDA devices (0 without a GPU; never fails) */
int tsph_device_count(int *count);

/* ---- particle system ---- */

/* Particle_system(h, kap, cs, rho0, visco, delta, dp) + Simulation_data
 * (src/SPH_particle_system.h:191-212, src/SPH_data.h:215-216).  `stream` is a
 * cudaStream_t or NULL for a stream owned by the system.  Fails with
 * TSPH_ERR_CUDA when no GPU is present. */
int tsph_create(const tsph_constants *c, const tsph_domain *d, int precision,
                void *stream, tsph_system **out);
int tsph_destroy(tsph_system *s);

/* Add_particle (src/SPH_particle_system.h:25-50) for n particles, plus the
 * mDBC ghost node of each wall particle (special.gnr, src/SPH_data.h:51,
 * pushed by the generators e.g. src/SPH_create.h:575-577).  gnr may be NULL
 * (DBC); for fluid entries it is ignored.  For boundary-integral walls
 * (TSPH_WALL_BT) the same array holds each wall particle's normal
 * (special.n, pushed by src/ALESPH_create.h:690-792).  Velocity of a wall
 * must be 0. */
int tsph_add_particles(tsph_system *s, int n, const int32_t *type,
                       const double *r, const double *v, const double *rho,
                       const double *p, const double *gnr);

int tsph_np(tsph_system *s, int *np);          /* live particles (particles.np) */
int tsph_grid(tsph_system *s, int *ncx, int *ncy);
int tsph_particle_mass(tsph_system *s, double *m);

/* Divide_To_Cells, src/SPH_find_pairs.h:5-42: grid of ncx x ncy cells of size
 * kh = kap*h, offset of = 0.273h, cell (x, y) -> id y + x*ncy. */
int tsph_divide_to_cells(tsph_system *s);
/* Clear_cells, src/SPH_find_pairs.h:74-92 (marks the cell lists stale) */
int tsph_clear_cells(tsph_system *s);
/* Particle_To_Cell, src/SPH_find_pairs.h:45-72: GPU counting sort by cell
 * (exact FP64 cell index, histogram, scan, stable scatter, SoA reorder).
 * On an FP32 system stepping with kept cells (the pair-record step) and
 * binned before, the cells and neighbour lists are kept when every particle
 * is within the skin of where it was binned (the decision is taken on the
 * device; the sort runs only when needed); the cell lists are then exact
 * again for every call that reads them (tsph_get_cells re-bins first). */
int tsph_particle_to_cell(tsph_system *s);
/* cells[c].cp as CSR in the reference's numbering: cell c holds
 * cell_list[cell_start[c] .. cell_start[c+1]), ascending particle index.
 * cell_start has ncx*ncy+1 entries, cell_list np entries. */
int tsph_get_cells(tsph_system *s, int32_t *cell_start, int32_t *cell_list);
/* Particle_To_Cell for callers that cannot allocate device memory.  This
 * entry point has no counterpart in the reference: it exists for callers whose
 * device memory comes only from their own pool (e.g. a host framework that
 * binds this library through its FFI) or whose time loop must not call
 * cudaMalloc/cudaFree (they synchronise the device).  The caller passes device
 * buffers: r_dev (double[2n] positions, x and y of each particle; 8-byte
 * aligned), cell_start_dev (int32[ncx*ncy+1]) and cell_list_dev (int32[n]),
 * both 4-byte aligned (misaligned pointers: TSPH_ERR_ARG before any work is
 * queued); the result is the reference's cells[c].cp as CSR (ascending
 * particle index in each cell) for the grid of Divide_To_Cells.
 * The counting sort's working memory is one static device array of about
 * 16.1 MB inside the library (held by every GPU that loads it until exit), so
 * n <= 1048576, ncx*ncy <= 1048576 and ncx, ncy <= 8192; larger sizes return
 * TSPH_ERR_ARG.  A cell may hold at most 4096 particles (a cell's ordering
 * cost grows with the square of its occupancy); a fuller cell returns
 * TSPH_ERR_ARG.  No allocation of any kind happens on the device.  The first
 * call on a device looks up that array's address and caches it for the
 * process; make it before any stream capture, and do not call this entry
 * point again after resetting the device (cudaDeviceReset) in the same
 * process.  Calls share the array and keep its last contents (each call clears
 * what must start at zero); calls that overlap on the GPU race, so the call
 * runs on `stream` (NULL = default stream) and waits for it before returning
 * (also when it fails after queueing work).
 * Particles outside the grid are left out and TSPH_ERR_ESCAPED is returned;
 * n_binned (may be NULL) receives the number of particles in the lists. */
int tsph_particle_to_cell_noalloc(const tsph_constants *c, const tsph_domain *d, int n,
                                  const double *r_dev, int32_t *cell_start_dev,
                                  int32_t *cell_list_dev, void *stream, int *n_binned);

/* Per-particle pair-set digest of the in-support pairs (0 < r <= 2h) over the
 * 3x3 cell block of each particle: count, sum and xor of the neighbours'
 * particle indices (reference numbering).  Arrays of np entries. */
int tsph_pair_digest(tsph_system *s, int32_t *count, int64_t *sum, int32_t *xor_);

/* Host-only (no GPU needed): the grid of Divide_To_Cells for (c, d) and the
 * exact cell-index tables the device uses in place of the FP64 division of
 * src/SPH_find_pairs.h:64-65.  bx[k] (k = 0..ncx) is the smallest double x,
 * mapped to a signed 64-bit integer that orders like the doubles (bits for
 * x >= +0, bits ^ 0x7fffffffffffffff for x < 0), whose cell index
 * (int)((x - x_0 + of)/kh) is >= k; by likewise.  Pass bx = by = NULL to get
 * ncx, ncy only. */
int tsph_grid_tables(const tsph_constants *c, const tsph_domain *d, int *ncx, int *ncy,
                     int64_t *bx, int64_t *by);

/* Density_to_pressure, src/SPH_pressure.h:65-89 (Tait EOS :7-21) */
int tsph_density_to_pressure(tsph_system *s);
/* mDBC_compute_density_mdbcGeo, src/SPH_mDBC.h:9-50 with
 * Kernel_density_approximation_MATRIX_mDBC, src/SPH_kernel_approx.h:1141-1343 */
int tsph_mdbc_density(tsph_system *s);
/* open boundaries (cases/inflowSlab_mDBC): a buffer zone, BufferZone(x0, xm,
 * y0, ym, nbl, v_b, orientation, btype) of src/SPH_inlet_outlet_data.h
 * pushed by DRAW_CreateInletY / DRAW_CreateOutletY (src/SPH_create.h:439-540);
 * its buffer particles are added with type btype (inlets 6-10, outlets
 * 11-15, src/SPH_defs.h:52-61).  Call before the first step.  A system with
 * zones runs tsph_step as the case's RUN loop (every zone's inlet or outlet
 * after the predictor) with per-function kernels. */
int tsph_add_buffer_zone(tsph_system *s, double x0, double xm, double y0, double ym, int nbl,
                         double vx, double vy, double ox, double oy, int btype);
/* room for the particles inlets create: extra fluid rows and extra particle
 * indices (defaults 65536 and 2^20); an inlet that would exceed them fails
 * with TSPH_ERR_NOMEM.  No counterpart in the reference. */
int tsph_set_zone_capacity(tsph_system *s, int extra_rows, int extra_ids);

/* Cases packed into one system (the batched workload; no counterpart in the
 * reference, which runs one case per process).  Every case is placed in the
 * system's frame scaled to the system's particle spacing (positions x
 * lambda_k, plus an offset), so that h, the mass, c0, dt and the other SPH
 * constants are the system's for every case; gravity scales with
 * 1/lambda_k and stays per case, as does RemoveParticlesOutOfDomain's box
 * (src/SPH_btdebug.h:4-31).  Per case k: x_range[2k..2k+1] = [lo, hi), the x
 * range of its grid columns (disjoint ranges: cases do not share a column;
 * a column between ranges goes to the nearest case), gravity[k], and
 * removal[4k..4k+3] =
 * (x_lo, x_hi, y_lo, y_hi): a fluid particle is erased when x < x_lo,
 * x > x_hi, y < y_lo or y > y_hi (the reference's thresholds, eps included,
 * in the system's frame).  Call after tsph_add_particles, before
 * tsph_particle_to_cell; ncases = 0 removes the table.  FP32 build, mDBC
 * walls, tsph_step only (the per-function force, corrector and removal calls
 * and tsph_save_checkpoint return TSPH_ERR_UNSUPPORTED on a system with a case
 * table); the fused step then uses the pair-record kernel, which reads each
 * window's case from its grid column, so the whole batch takes one launch per
 * kernel per step. */
int tsph_set_cases(tsph_system *s, int ncases, const double *x_range, const double *gravity,
                   const double *removal);
/* BZ_Integrate_inlet / BZ_Integrate_outlet, src/SPH_buffer_zones.h:10-206 */
int tsph_bz_inlet(tsph_system *s, int zone, double dt);
int tsph_bz_outlet(tsph_system *s, int zone, double dt);
/* BT_compute_density_BTGeo, src/SPH_BT.h:9-50 with
 * Kernel_density_approximation_BT_update, src/SPH_kernel_approx.h:1838-1953:
 * the density of boundary-integral wall particles */
int tsph_bt_density(tsph_system *s);
/* Compute_Forces: src/SPH_interaction.h:8-149 (TSPH_WALL_MDBC),
 * src/SPH_interactionDBC.h:8-155 (TSPH_WALL_DBC) or
 * src/SPH_interactionBT.h:8-194 (TSPH_WALL_BT, walls with normals) */
int tsph_compute_forces(tsph_system *s, int wall_model);
/* Integrate_SymplecticPredictor / Corrector, src/SPH_integration.h:266-309 */
int tsph_symplectic_predictor(tsph_system *s, double dt);
int tsph_symplectic_corrector(tsph_system *s, double dt);
/* RemoveParticlesOutOfDomain, src/SPH_btdebug.h:4-31 */
int tsph_remove_out_of_domain(tsph_system *s, int *removed);

/* nsteps bodies of SPH_simulation::RUN (cases/damBreakLong_mDBC/
 * SPH_simulationSymplectic.h:59-118 for mDBC, cases/stillWater_DBC/
 * SPH_simulationSymplectic.h:58-118 for DBC, cases/damBreakLong_BT/
 * SPH_simulationSymplectic.h for BT walls) as fused kernels replayed from a
 * CUDA graph.  Requires tsph_particle_to_cell to have been called once (INIT,
 * :41-45).  Leaves the state the reference has after the same steps; its
 * pressure (p = EOS(rho), which the steps form inside their pair records) is
 * written to the state by the next call that reads or replaces the state
 * (download, probes, per-function calls, save), not after every call, so a
 * time loop of tsph_step calls runs no equation-of-state launch between
 * steps. */
int tsph_step(tsph_system *s, int wall_model, double dt, int nsteps);

/* state transfer in the reference's order; `fields` is a TSPH_F_* mask */
int tsph_download(tsph_system *s, int fields, const tsph_host_state *out);
int tsph_upload(tsph_system *s, int fields, const tsph_host_state *in);
/* Pipelined download (no counterpart in the reference, whose state lives in
 * host memory): tsph_download_async exports r, v, a, rho, drho and p (other
 * fields: TSPH_ERR_ARG) into a staging set of its own on the system's stream
 * and starts the device-to-host copies on a copy stream, then returns; the
 * copies run beside the calls that follow (the next upload and step).
 * tsph_download_wait blocks until they are done.  Until then the host
 * buffers (pinned memory for a true overlap) must stay valid and unread.  At
 * most one download is in flight: a second tsph_download_async first waits
 * for the one before.  A state with erased particles is downloaded
 * synchronously (its rows are compacted on the host). */
int tsph_download_async(tsph_system *s, int fields, const tsph_host_state *out);
int tsph_download_wait(tsph_system *s);
/* Staged upload (no counterpart in the reference): the host-to-device copies
 * of r, v, a, rho, drho and p (other fields: TSPH_ERR_ARG) start on a copy
 * stream of their own, beside the work already enqueued (a step in flight),
 * and the call returns; the next tsph_particle_to_cell applies them and bins
 * the new state.  Between the two, only tsph_download_async / _wait and
 * tsph_health may be called (tsph_download and tsph_upload return
 * TSPH_ERR_STATE; calls that need cell lists find them stale).  Every
 * particle index must still be live (no erased particles: the rows are taken
 * as indices 0..n-1); otherwise the upload is dropped and TSPH_HEALTH_UPLOAD
 * is raised.  The host buffers (pinned for a true overlap) must stay valid
 * until tsph_particle_to_cell returns. */
int tsph_upload_async(tsph_system *s, int fields, const tsph_host_state *in);
/* wait for the system's stream */
int tsph_sync(tsph_system *s);
/* device health word (TSPH_HEALTH_*), optionally cleared */
int tsph_health(tsph_system *s, uint32_t *flags, int clear);
/* number of kernels the library launched for this system (no counterpart in
 * the reference): eager launches, the kernels of every CUDA-graph step
 * launched, and those of the conditional re-binning each time it ran on the
 * device; optionally reset to zero */
int tsph_kernel_launches(tsph_system *s, long long *count, int reset);

/* Global reductions in FP64 over fluid particles: total mass, kinetic energy
 * sum(0.5 m |v|^2) (the harness-side Total_kinetic_energy the still-water
 * driver calls), and momentum. out[0..3] = mass, ekin, px, py. */
int tsph_fluid_totals(tsph_system *s, double out[4]);

/* ---- probes of the case drivers (cases/damBreakLong_mDBC/
 * SPH_simulationSymplectic.h:156-199), on the current state and cells.
 * Water_Elevation / Water_Elevation_inverse (src/SPH_water_level.h:84-150)
 * at n gauges: from (x[k], y0[k]) upwards (inverse[k] = 0) or downwards
 * (inverse[k] = 1; inverse may be NULL) with the reference's growing sampling
 * step dp * 5e-5 * i, to the first height where the kernel volume sum m W /
 * rho drops to (rises to) 0.5; out[k] = that level, NaN if never reached. */
int tsph_water_level(tsph_system *s, int n, const double *x, const double *y0,
                     const int32_t *inverse, double *out);
/* Kernel_velocity_approximation_TEST (src/testing.h:6-149) at n points
 * xy[2k], xy[2k+1]: out[4k..4k+3] = Shepard {rho, p, vx, vy} (0 where the
 * kernel volume is <= 0.5); Pressure_in_point (src/SPH_measure_pressure.h:6-15)
 * is out[4k+1]. */
int tsph_point_fields(tsph_system *s, int n, const double *xy, double *out);
/* water front: the largest x of the live fluid with y <= y_max (NaN if
 * none).  No counterpart in the reference, which records no front. */
int tsph_water_front(tsph_system *s, double y_max, double *x_front);

/* Kernel timing of the system's calls, for the roofline report.  With
 * profiling on, tsph_step runs its kernels eagerly (no graph) with CUDA events
 * around every launch on the system's stream; tsph_profile returns the sums
 * since the last reset.  Off by default (graph replay, no events). */
typedef struct {
    double pair_us;      /* pair-loop + fused integrator kernels (the pair
                            records of variant 2 count as other)          */
    int pair_launches;
    double sort_us;      /* cell keys, scan, stable scatter                */
    int sort_launches;
    double mdbc_us;      /* ghost-node density                            */
    int mdbc_launches;
    double other_us;     /* everything else (EOS, predictor, ...)         */
    int other_launches;
} tsph_profile_t;
/* Variant of the FP32 pair kernel (TSPH_N_TILE_SHAPES of them):
 * 0 = one CTA per 128 targets staging 608 neighbours with 36 list entries per
 *     target, 1 = the same with 512 and 44 (for h ~ 1.5 dp),
 * 2 = pair records: a pass forms every particle's neighbour-side values and
 *     the table of each chunk's windows once, then one CTA per 128 targets
 *     stages each window's record ranges with bulk copies (528 staged
 *     neighbours, 38 list entries per target).
 * tsph_autotune times every variant on the current particles (a warm-up and
 * 20 timed forces passes each, the median kept; the state is left as it was)
 * and keeps the fastest; the first tsph_step does this by itself.
 * us (may be NULL) receives TSPH_N_TILE_SHAPES median times in microseconds.
 * No counterpart in the reference. */
#define TSPH_N_TILE_SHAPES 3
int tsph_autotune(tsph_system *s, int32_t *shape, double us[TSPH_N_TILE_SHAPES]);
int tsph_set_tile_shape(tsph_system *s, int shape);
/* the variant in use (-1 before the first tsph_step or tsph_autotune) */
int tsph_get_tile_shape(tsph_system *s, int32_t *shape);
int tsph_set_profiling(tsph_system *s, int on);

/* ---- the particle graph of the learned surrogate (no counterpart in the
 * reference).  Nodes: walls first, then the live fluid in the system's sorted
 * order; edges: the pairs within the kernel support (0 < r <= 2h).  All
 * arrays are DEVICE pointers with room for `capacity` nodes: pos (double2),
 * vel (float2), srho (rho - rho0), wall (1 for walls), id (particle index),
 * deg, nbr (k_slots per node, unused slots -1); acc (float2) and rate (float)
 * may be NULL, else they receive the rates of the last forces pass, a and
 * d(rho)/dt (zero for walls).  TSPH_ERR_UNSUPPORTED if a node has more than
 * k_slots neighbours. */
int tsph_export_graph(tsph_system *s, int k_slots, int capacity, void *pos, void *vel,
                      float *srho, float *wall, int32_t *id, int32_t *deg, int32_t *nbr,
                      void *acc, float *rate, int32_t *n_nodes, int32_t *n_wall);
/* the surrogate's update of the fluid over a window of k steps (k_dt = k dt),
 * from y (device, 3 floats per node of the last export), with a, drho/dt
 * those of the last forces pass and r = 1 if flags has TSPH_UPDATE_RATES:
 *   phase 0 (explicit):  v_new = v + r k_dt a + u_scale (y0, y1),
 *                        rho_new = rho + r k_dt drho/dt + s_scale y2,
 *                        r += k_dt (v + v_new) / 2;
 *   phase 1 (kick):      v_new as in phase 0; rho and r unchanged (the cell
 *                        lists stay valid, for a forces pass with v_new);
 *   phase 2 (drift, after a kick and a forces pass):
 *                        rho += r k_dt drho/dt + s_scale y2 with the rate of
 *                        that pass, r += k_dt (v_start + v_new) / 2.
 * With TSPH_UPDATE_ZERO_MOMENTUM, (y0, y1) less their mean over the fluid
 * nodes is used: the correction carries no momentum.  Phases 0 and 1 record,
 * per particle, the start-of-window terms of the window check
 * (tsph_window_check).  The cell lists are stale after phases 0 and 2. */
enum { TSPH_UPDATE_RATES = 1, TSPH_UPDATE_ZERO_MOMENTUM = 2 };
int tsph_apply_update(tsph_system *s, const float *y, double u_scale, double s_scale,
                      double k_dt, int flags, int phase);
/* the per-window check of a surrogate window, after a forces pass at the
 * window's end state: against the trapezoidal rule of the SPH rates at both
 * ends, rho_c = rho_0 + k_dt (drho_0 + drho_1) / 2 and
 * v_c = v_0 + k_dt (a_0 + a_1) / 2, per fluid particle,
 *   out[0] = max |rho - rho_c| / rho0,  out[1] = rms |rho - rho_c| / rho0,
 *   out[2] = |sum m (v - v_c)| / (M g k_dt)  (momentum, against gravity's
 *            impulse on the fluid mass M over the window),
 *   out[3] = the number of fluid particles checked,
 *   out[4] = the particle index of the largest density error. */
int tsph_window_check(tsph_system *s, double k_dt, double out[5]);
/* the CUDA stream the system's kernels run on (the caller's, or the one the
 * system created when given NULL): work of other libraries on the same
 * buffers (the surrogate's network, for one) must be ordered with it.  No
 * counterpart in the reference. */
int tsph_get_stream(tsph_system *s, void **stream);
/* a device-side copy of the whole particle state (the start of a surrogate
 * window) and its restoration (the plain-step fallback). */
int tsph_state_save(tsph_system *s);
int tsph_state_restore(tsph_system *s);

/* ---- the surrogate's graph network (no counterpart in the reference): a
 * two-layer message-passing network of hidden width 64 over an exported
 * particle graph, predicting per node (du, dv, d(rho - rho0)) over a window of
 * k SPH steps in units of the graph's scales.  Forward, loss gradient and Adam
 * run on the device; parameters are FP32, in the order of
 * oracle/gnn_oracle.py (tsph_gnn_n_params of them). */
typedef struct tsph_gnn tsph_gnn;
typedef struct {
    const void *pos;           /* double2 per node (device) */
    const void *vel;           /* float2 per node (device) */
    const float *srho, *wall;  /* rho - rho0, wall flag (device) */
    const int32_t *deg, *nbr;  /* neighbour table, k_slots per node (device) */
    int32_t n_nodes, k_slots;
    double h, u_scale, s_scale;  /* edge length, velocity and density scales */
} tsph_gnn_graph;
int tsph_gnn_n_params(void);
int tsph_gnn_create(int capacity, void *stream, tsph_gnn **out);
int tsph_gnn_destroy(tsph_gnn *g);
int tsph_gnn_set_params(tsph_gnn *g, const float *host);  /* also resets Adam */
int tsph_gnn_get_params(tsph_gnn *g, float *host);
int tsph_gnn_get_grads(tsph_gnn *g, float *host);
/* y (device, 3 per node) may be NULL */
int tsph_gnn_forward(tsph_gnn *g, const tsph_gnn_graph *graph, float *y);
/* the same network's forward pass for the rollout: BF16 weights and
 * activations on the tensor cores with FP32 accumulation, the edge sums in
 * FP32 with the hardware tanh in SiLU; y (device, n x 3) is required.  Its
 * outputs differ from tsph_gnn_forward's by the BF16 rounding (about 1 %). */
int tsph_gnn_infer(tsph_gnn *g, const tsph_gnn_graph *graph, float *y);
/* forward, mean squared error against target (device, 3 per node) over the
 * fluid nodes, gradient into the network's gradient buffer */
int tsph_gnn_loss_grad(tsph_gnn *g, const tsph_gnn_graph *graph, const float *target,
                       double *loss);
int tsph_gnn_adam(tsph_gnn *g, double lr, double beta1, double beta2, double eps);

/* ---- output and restart
 * write_to_ASCII_VTK (src/SPH_data_to_vtk.h:4-51): the same POLYDATA file
 * (points, type, pressure, density, velocity) in the reference's order. */
int tsph_write_vtk(tsph_system *s, const char *path);
/* binary checkpoint of the live particles (state, rates, types, ghost nodes,
 * buffer zones and their capacities, constants, domain, precision, tile
 * shape; no counterpart in the reference)
 * and a new system restarted from it: stepping it continues the saved run
 * bit for bit.  Saving re-bins a system that steps with kept neighbour lists
 * (tile shape 2), so the saved run and the restarted one go on from the same
 * binning. */
int tsph_save_checkpoint(tsph_system *s, const char *path);
int tsph_load_checkpoint(const char *path, void *stream, tsph_system **out);
int tsph_get_profile(tsph_system *s, tsph_profile_t *out, int reset);

/* ==================================================================
 * Riemann / ALE-SPH (cases/ALESPH_dambreakLong/MUSCL.h path): leap-frog in
 * omega (volume), omega*rho and omega*v (src/RALESPH_integration.h), the
 * one-sided MUSCL gradients (src/_testMUSCL_gradientApprox.h) and the flux
 * loop with the linearised Riemann solver (src/_testMUSCL_interaction.h,
 * src/ALESPH_riemann_solver.h).  BT walls carry a normal each (special.n).
 * FP32 fluxes, FP64 integration of the conserved variables.
 * ================================================================== */
typedef struct tsph_ale_system tsph_ale_system;

/* interface states of the flux loop: as the reference's MUSCL.h driver
 * computes them (MUSCL_final adds 0.5 dt/dx (F(W_L) - F(W_L)) = 0 and the
 * neighbour state carries the active particle's velocity,
 * src/_testMUSCL_interaction.h:185, src/_testMUSCL_schemes.h:78-88); the
 * superbee-limited MUSCL states of both particles (no counterpart in the
 * reference); or the first-order fluxes of the SPH_simulationINT.h driver
 * (Compute_Forces(Particle_system&), src/RALESPH_interaction.h:12-289: both
 * particles' own states, limited Riemann density, linear wall pressure; no
 * gradient pass) */
enum { TSPH_ALE_AS_WRITTEN = 0, TSPH_ALE_MUSCL = 1, TSPH_ALE_FIRST_ORDER = 2 };

/* host view; any pointer may be NULL.  grad: 12 per particle (rho, vx, vy
 * forward x/y, then backward x/y: special.grad*F, grad*B), valid from
 * tsph_ale_gradient until the particles are next re-binned.  p is the
 * reference's p: the equation of state of the density that the last flux pass
 * used (Density_to_pressure runs before the fluxes, not after the leap-frog) */
typedef struct {
    double *r, *v, *rho, *p;
    double *omega, *omegarho, *omegav, *domega, *domegarho, *domegav, *grad;
    int32_t *index, *type;
} tsph_ale_host_state;

enum {
    TSPH_ALE_F_R = 1 << 0, TSPH_ALE_F_V = 1 << 1, TSPH_ALE_F_RHO = 1 << 2, TSPH_ALE_F_P = 1 << 3,
    TSPH_ALE_F_OMEGA = 1 << 4, TSPH_ALE_F_OMEGARHO = 1 << 5, TSPH_ALE_F_OMEGAV = 1 << 6,
    TSPH_ALE_F_RATES = 1 << 7, TSPH_ALE_F_GRAD = 1 << 8, TSPH_ALE_F_INDEX = 1 << 9,
    TSPH_ALE_F_TYPE = 1 << 10
};

/* Particle_system + Simulation_data for the ALE path */
int tsph_ale_create(const tsph_constants *c, const tsph_domain *d, void *stream,
                    tsph_ale_system **out);
int tsph_ale_destroy(tsph_ale_system *s);
/* ALESPH_Add_particle (src/SPH_particle_system.h:51-108: omega = dp^2,
 * omega*v, omega*rho) for n particles; `normal` (2n, may be NULL for fluid)
 * is special.n of the wall particles (src/ALESPH_create.h:719) */
int tsph_ale_add_particles(tsph_ale_system *s, int n, const int32_t *type, const double *r,
                           const double *v, const double *rho, const double *p,
                           const double *normal);
int tsph_ale_set_scheme(tsph_ale_system *s, int scheme);
/* Kept cells for tsph_ale_step and tsph_ale_particle_to_cell (on by
 * default; no counterpart in the reference, whose RUN loop re-bins and sorts
 * every step, cases/ALESPH_dambreakLong/MUSCL.h:80-140): the cells of the
 * last binning stay while every fluid particle is within 0.95 (kh - 2h) / 2
 * of where it was binned and none left the domain; part two then runs in
 * place and the sort only when one did.  The pair sums are the same up to FP32 summation
 * order; off, every step sorts into the reference's cell order (needs kh >
 * 2h to be on). */
int tsph_ale_set_keep_cells(tsph_ale_system *s, int on);
/* sorts run by tsph_ale_step on kept cells since the system was built */
int tsph_ale_sort_count(tsph_ale_system *s, long long *n);
int tsph_ale_np(tsph_ale_system *s, int *np);
/* Divide_To_Cells + Particle_To_Cell, src/SPH_find_pairs.h:5-72 */
int tsph_ale_divide_to_cells(tsph_ale_system *s);
int tsph_ale_particle_to_cell(tsph_ale_system *s);
/* Kernel_gradient_approx, src/_testMUSCL_gradientApprox.h:10-231 */
int tsph_ale_gradient(tsph_ale_system *s);
/* Compute_Forces(particles, dt), src/_testMUSCL_interaction.h:13-324 */
int tsph_ale_forces(tsph_ale_system *s, double dt);
/* Integrate_LeapFrog_partOne / partTwo, src/RALESPH_integration.h:10-107 */
int tsph_ale_leapfrog_one(tsph_ale_system *s, double dt);
int tsph_ale_leapfrog_two(tsph_ale_system *s, double dt, int step);
/* nsteps bodies of SPH_simulation::RUN of cases/ALESPH_dambreakLong/MUSCL.h:82-137
 * (steps step0+1 .. step0+nsteps); the gradient pass runs only for
 * TSPH_ALE_MUSCL (the as-written fluxes do not depend on it) */
int tsph_ale_step(tsph_ale_system *s, double dt, int step0, int nsteps);
int tsph_ale_download(tsph_ale_system *s, int fields, const tsph_ale_host_state *out);
int tsph_ale_upload(tsph_ale_system *s, int fields, const tsph_ale_host_state *in);
/* Pipelined transfers of r, v and rho (TSPH_ALE_F_R | _V | _RHO; other
 * fields TSPH_ERR_ARG), as tsph_download_async / tsph_download_wait /
 * tsph_upload_async for the WCSPH system (no counterpart in the reference,
 * whose state lives in host memory).  tsph_ale_download_async exports into a
 * staging set of its own and starts the device-to-host copies on a copy
 * stream; tsph_ale_download_wait blocks until they are done (host buffers,
 * pinned for a true overlap, valid and unread until then; with removed
 * particles the download is synchronous).  tsph_ale_upload_async starts the
 * host-to-device copies on a copy stream beside the work in flight; the next
 * tsph_ale_particle_to_cell applies them (only if every particle is still
 * live, else TSPH_HEALTH_UPLOAD and nothing changes) and bins the state;
 * until then the calls that read or write the state return TSPH_ERR_STATE. */
int tsph_ale_download_async(tsph_ale_system *s, int fields, const tsph_ale_host_state *out);
int tsph_ale_download_wait(tsph_ale_system *s);
int tsph_ale_upload_async(tsph_ale_system *s, int fields, const tsph_ale_host_state *in);
int tsph_ale_sync(tsph_ale_system *s);
int tsph_ale_health(tsph_ale_system *s, uint32_t *flags, int clear);

#ifdef __cplusplus
}
#endif
#endif /* TSPH_H */
