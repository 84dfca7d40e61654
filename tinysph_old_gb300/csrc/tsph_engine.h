// tsph_engine.h -- host-side interface between the C ABI (tsph_api.cpp) and
// the precision-specific engines (tsph_engine_f32.cu / tsph_engine_f64.cu).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace tsph {

// Everything the device side needs, prepared on the host.
struct HostSetup {
    // SPH_constants (src/SPH_data.h:124-140)
    double h, kap, cs, rho0, visco, delta, dp, m, g;
    // Simulation_data (padded domain)
    double x0, xm, y0, ym;
    // grid (Divide_To_Cells, src/SPH_find_pairs.h:5-42)
    double kh, of;
    int ncx, ncy;
    std::vector<long long> bx, by;  // ordered-int64 lower bounds of each cell index, n+1
    std::vector<double> ox, oy;     // cell origins
    // particles in the reference's order
    std::vector<int> type;
    std::vector<double> r, v, a, rho, drho, p, gnr;  // r, v, a, gnr interleaved (x, y)
    std::vector<uint8_t> has_gnr;
    // open boundaries: per zone orientation x, y; x0, y0, xm, ym; nbl; bl, bh;
    // btype; v_b x, y (BufferZone, src/SPH_inlet_outlet_data.h), and the
    // room for particles the inlets create
    std::vector<double> zones;
    int extra_rows = 65536, extra_ids = 1 << 20;
    // cases packed into one system (tsph_set_cases): per case the x range
    // [lo, hi) of its grid columns, its gravity, and its removal thresholds
    // (x_lo, x_hi, y_lo, y_hi: removed when x < x_lo, x > x_hi, y < y_lo or
    // y > y_hi); empty for a single case
    std::vector<double> case_x, case_g, case_box;
};

struct Profile {
    double us[4] = {0, 0, 0, 0};
    int launches[4] = {0, 0, 0, 0};
};

enum { CAT_PAIR = 0, CAT_SORT = 1, CAT_MDBC = 2, CAT_OTHER = 3 };

class EngineBase {
  public:
    virtual ~EngineBase() {}
    // all calls return a TSPH_* status and set `err` on failure
    virtual int init(const HostSetup &hs, void *stream, std::string &err) = 0;
    virtual int particle_to_cell(std::string &err) = 0;
    virtual int density_to_pressure(std::string &err) = 0;
    virtual int mdbc_density(std::string &err) = 0;
    virtual int bt_density(std::string &err) = 0;
    virtual int compute_forces(int model, std::string &err) = 0;
    virtual int predictor(double dt, std::string &err) = 0;
    virtual int corrector(double dt, std::string &err) = 0;
    virtual int remove_out_of_domain(int *removed, std::string &err) = 0;
    virtual int step(int model, double dt, int nsteps, std::string &err) = 0;
    // state in the reference's order: the engine fills per-index staging and
    // reports which indices are alive (removed particles are not)
    virtual int download(int mask, double *r, double *v, double *a, double *rho, double *drho,
                         double *p, int32_t *index, int32_t *type, std::string &err) = 0;
    virtual int download_async(int mask, double *r, double *v, double *a, double *rho,
                               double *drho, double *p, std::string &err) = 0;
    virtual int download_wait(std::string &err) = 0;
    virtual int upload_async(int mask, const double *r, const double *v, const double *a,
                             const double *rho, const double *drho, const double *p,
                             std::string &err) = 0;
    virtual int upload(int mask, const double *r, const double *v, const double *a,
                       const double *rho, const double *drho, const double *p,
                       std::string &err) = 0;
    virtual int get_cells(int32_t *cell_start, int32_t *cell_list, std::string &err) = 0;
    virtual int pair_digest(int32_t *count, int64_t *sum, int32_t *xr, std::string &err) = 0;
    virtual int np_live(int *np, std::string &err) = 0;
    virtual int kernel_launches(long long *count, int reset, std::string &err) = 0;
    virtual int health(uint32_t *flags, int clear, std::string &err) = 0;
    virtual int totals(double out[4], std::string &err) = 0;
    virtual int water_level(int n, const double *x, const double *y0, const int32_t *inverse,
                            double *out, std::string &err) = 0;
    virtual int point_fields(int n, const double *xy, double *out, std::string &err) = 0;
    virtual int water_front(double y_max, double *x, std::string &err) = 0;
    virtual int autotune(int *choice, double *us, std::string &err) = 0;
    virtual int set_tile_shape(int shape, std::string &err) = 0;
    virtual int tile_shape() const = 0;
    // the particle graph and the surrogate's window update (device pointers)
    virtual int export_graph(int K, int cap, double2 *pos, float2 *vel, float *srho, float *wall,
                             int32_t *id, int32_t *deg, int32_t *nbr, float2 *acc, float *rate,
                             int *n_nodes, int *n_wall, std::string &err) = 0;
    virtual int apply_update(const float *y, double su, double ss, double kdt, bool add_rates,
                             bool zero_momentum, int phase, std::string &err) = 0;
    virtual int window_check(double kdt, double out[5], std::string &err) = 0;
    virtual int bz_inlet(int zone, double dt, std::string &err) = 0;
    virtual int bz_outlet(int zone, double dt, std::string &err) = 0;
    virtual int state_save(std::string &err) = 0;
    virtual int state_restore(std::string &err) = 0;
    virtual int sync(std::string &err) = 0;
    virtual void *stream() const = 0;
    virtual void set_profiling(bool on) = 0;
    virtual Profile profile(bool reset) = 0;
    virtual bool cells_valid() const = 0;
    // cells kept over several steps (kept neighbour lists) re-binned at the
    // current positions; nothing when they are the current positions' cells
    virtual int settle_cells(std::string &err) = 0;
    virtual void invalidate_cells() = 0;
};

// message returned by tsph_last_error() for the calling thread
void set_last_error(const std::string &msg);

EngineBase *make_engine_f32();
EngineBase *make_engine_f64();

}  // namespace tsph
