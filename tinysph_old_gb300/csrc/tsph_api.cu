// tsph_api.cu -- the extern "C" boundary (include/tsph.h): argument checks,
// the reference's grid arithmetic (Divide_To_Cells) and its exact cell-index
// tables, and dispatch to the FP32 or FP64 engine.
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/tsph.h"
#include "tsph_engine.h"
#include "tsph_grid_host.h"
#include "tsph_internal.cuh"

using tsph::EngineBase;
using tsph::HostSetup;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

using tsph::cell_lower_bound;

}  // namespace

namespace tsph {
void set_last_error(const std::string &msg) { g_err = msg; }
}  // namespace tsph

#include "tsph_system.h"

static int ensure_engine(tsph_system *s) {
    if (!s->divided) return fail(TSPH_ERR_STATE, "call tsph_divide_to_cells first");
    if (s->eng && !s->stale_engine) return TSPH_OK;
    if (s->hs.zones.empty())
        for (int t : s->hs.type)
            if (t != TSPH_FLUID && t != TSPH_WALL)
                return fail(TSPH_ERR_UNSUPPORTED, "particle type " + std::to_string(t) +
                                                      " needs a buffer zone (tsph_add_buffer_zone)");
    std::unique_ptr<EngineBase> e(s->precision == TSPH_PREC_FP64 ? tsph::make_engine_f64()
                                                                  : tsph::make_engine_f32());
    std::string err;
    s->eng.reset();
    int rc = e->init(s->hs, s->stream, err);
    if (rc) return fail(rc, err);
    e->set_profiling(s->profiling);
    s->eng = std::move(e);
    s->stale_engine = false;
    return TSPH_OK;
}

#define NEED(s)                                                        \
    do {                                                               \
        if (!(s)) return fail(TSPH_ERR_ARG, "null system handle");     \
    } while (0)

#define ENGINE(s)                                                      \
    do {                                                               \
        int rc_ = ensure_engine(s);                                    \
        if (rc_) return rc_;                                           \
    } while (0)

#define RUN(expr)                                                      \
    do {                                                               \
        std::string err_;                                              \
        int rc_ = (expr);                                              \
        if (rc_) return fail(rc_, err_);                               \
    } while (0)

extern "C" {

int tsph_abi_version(void) { return TSPH_ABI_VERSION; }

const char *tsph_last_error(void) { return g_err.c_str(); }

const char *tsph_status_string(int status) {
    switch (status) {
    case TSPH_OK: return "ok";
    case TSPH_ERR_ARG: return "invalid argument";
    case TSPH_ERR_CUDA: return "CUDA error";
    case TSPH_ERR_STATE: return "call out of order";
    case TSPH_ERR_NOMEM: return "out of memory";
    case TSPH_ERR_NUMERIC: return "NaN or Inf in the state";
    case TSPH_ERR_DENSITY: return "density out of range";
    case TSPH_ERR_ESCAPED: return "particle left the grid";
    case TSPH_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

int tsph_device_count(int *count) {
    if (!count) return fail(TSPH_ERR_ARG, "null count");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return TSPH_OK;
}

int tsph_create(const tsph_constants *c, const tsph_domain *d, int precision, void *stream,
                tsph_system **out) {
    if (!c || !d || !out) return fail(TSPH_ERR_ARG, "null argument");
    *out = nullptr;
    if (precision != TSPH_PREC_FP32 && precision != TSPH_PREC_FP64)
        return fail(TSPH_ERR_ARG, "precision must be TSPH_PREC_FP32 or TSPH_PREC_FP64");
    if (!(c->h > 0) || !(c->kap > 0) || !(c->dp > 0) || !(c->cs > 0) || !(c->rho0 > 0))
        return fail(TSPH_ERR_ARG, "h, kap, dp, cs and rho0 must be positive");
    if (!(d->x_m > d->x_0) || !(d->y_m > d->y_0)) return fail(TSPH_ERR_ARG, "empty domain");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(TSPH_ERR_CUDA, "no CUDA device available");
    }
    tsph_system *s = new tsph_system();
    HostSetup &hs = s->hs;
    // Particle_system constructor, src/SPH_particle_system.h:191-212
    hs.h = c->h;
    hs.kap = c->kap;
    hs.cs = c->cs;
    hs.rho0 = c->rho0;
    hs.dp = c->dp;
    hs.g = 9.81;
    hs.m = c->rho0 / (1 / c->dp * 1 / c->dp);
    hs.visco = c->visco;
    hs.delta = c->delta;
    hs.x0 = d->x_0;
    hs.xm = d->x_m;
    hs.y0 = d->y_0;
    hs.ym = d->y_m;
    s->precision = precision;
    s->stream = stream;
    *out = s;
    return TSPH_OK;
}

int tsph_destroy(tsph_system *s) {
    delete s;
    return TSPH_OK;
}

int tsph_add_particles(tsph_system *s, int n, const int32_t *type, const double *r,
                       const double *v, const double *rho, const double *p, const double *gnr) {
    NEED(s);
    if (n < 0) return fail(TSPH_ERR_ARG, "negative count");
    if (n == 0) return TSPH_OK;
    if (!type || !r || !rho) return fail(TSPH_ERR_ARG, "type, r and rho are required");
    for (int i = 0; i < n; i++) {
        if (type[i] < 0 || type[i] > 255)
            return fail(TSPH_ERR_ARG, "particle type " + std::to_string(type[i]) +
                                          " (fluid 0, wall 1, buffer types 2-255)");
        if (type[i] == TSPH_WALL && v && (v[2 * i] != 0.0 || v[2 * i + 1] != 0.0))
            return fail(TSPH_ERR_UNSUPPORTED, "moving walls are not on this path (wall v must be 0)");
        if (!std::isfinite(r[2 * i]) || !std::isfinite(r[2 * i + 1]) || !std::isfinite(rho[i]))
            return fail(TSPH_ERR_ARG, "non-finite position or density");
    }
    HostSetup &hs = s->hs;
    // keep the evolved state when particles are appended to a running system
    if (s->eng && !s->stale_engine) {
        int np = 0;
        std::string err;
        int rc = s->eng->np_live(&np, err);
        if (rc) return fail(rc, err);
        if (np != (int)hs.type.size())
            return fail(TSPH_ERR_STATE, "cannot append particles after removals");
        std::vector<double> R(2 * np), V(2 * np), A(2 * np), RHO(np), DRHO(np), P(np);
        rc = s->eng->download(63, R.data(), V.data(), A.data(), RHO.data(), DRHO.data(), P.data(),
                              nullptr, nullptr, err);
        if (rc) return fail(rc, err);
        hs.r = R;
        hs.v = V;
        hs.a = A;
        hs.rho = RHO;
        hs.drho = DRHO;
        hs.p = P;
    }
    for (int i = 0; i < n; i++) {
        hs.type.push_back(type[i]);
        hs.r.push_back(r[2 * i]);
        hs.r.push_back(r[2 * i + 1]);
        hs.v.push_back(v ? v[2 * i] : 0.0);
        hs.v.push_back(v ? v[2 * i + 1] : 0.0);
        hs.a.push_back(0.0);
        hs.a.push_back(0.0);
        hs.rho.push_back(rho[i]);
        hs.drho.push_back(0.0);
        hs.p.push_back(p ? p[i] : 0.0);
        const bool g = gnr && type[i] == TSPH_WALL;
        hs.gnr.push_back(g ? gnr[2 * i] : 0.0);
        hs.gnr.push_back(g ? gnr[2 * i + 1] : 0.0);
        hs.has_gnr.push_back(g ? 1 : 0);
    }
    s->stale_engine = true;
    return TSPH_OK;
}

int tsph_np(tsph_system *s, int *np) {
    NEED(s);
    if (!np) return fail(TSPH_ERR_ARG, "null np");
    if (!s->eng || s->stale_engine) {
        *np = (int)s->hs.type.size();
        return TSPH_OK;
    }
    RUN(s->eng->np_live(np, err_));
    return TSPH_OK;
}

int tsph_grid(tsph_system *s, int *ncx, int *ncy) {
    NEED(s);
    if (!s->divided) return fail(TSPH_ERR_STATE, "call tsph_divide_to_cells first");
    if (ncx) *ncx = s->hs.ncx;
    if (ncy) *ncy = s->hs.ncy;
    return TSPH_OK;
}

int tsph_particle_mass(tsph_system *s, double *m) {
    NEED(s);
    if (!m) return fail(TSPH_ERR_ARG, "null m");
    *m = s->hs.m;
    return TSPH_OK;
}

// grid dimensions and exact cell-index tables (Divide_To_Cells,
// src/SPH_find_pairs.h:5-42, and the index of :64-65)
static int make_grid(HostSetup &hs) {
    const double kh = hs.kap * hs.h;
    const double of = hs.h * 0.273;
    const double qx = (hs.xm - hs.x0 + of) / kh, qy = (hs.ym - hs.y0 + of) / kh;
    if (!(qx < 1e7) || !(qy < 1e7)) return fail(TSPH_ERR_ARG, "grid too large");
    const int ncx = (int)qx + 1;
    const int ncy = (int)qy + 1;
    if (ncy < 4 || ncx < 1) return fail(TSPH_ERR_UNSUPPORTED, "grid needs at least 4 cells in y");
    if ((long long)ncx * ncy > 200000000LL) return fail(TSPH_ERR_ARG, "grid too large");
    hs.kh = kh;
    hs.of = of;
    hs.ncx = ncx;
    hs.ncy = ncy;
    hs.bx.resize(ncx + 1);
    hs.by.resize(ncy + 1);
    for (int k = 0; k <= ncx; k++) hs.bx[k] = cell_lower_bound(k, hs.x0, of, kh);
    for (int k = 0; k <= ncy; k++) hs.by[k] = cell_lower_bound(k, hs.y0, of, kh);
    hs.ox.resize(ncx);
    hs.oy.resize(ncy);
    for (int k = 0; k < ncx; k++) hs.ox[k] = (hs.x0 - of) + k * kh;
    for (int k = 0; k < ncy; k++) hs.oy[k] = (hs.y0 - of) + k * kh;
    return TSPH_OK;
}

int tsph_grid_tables(const tsph_constants *c, const tsph_domain *d, int *ncx, int *ncy,
                     int64_t *bx, int64_t *by) {
    if (!c || !d || !ncx || !ncy) return fail(TSPH_ERR_ARG, "null argument");
    if (!(c->h > 0) || !(c->kap > 0)) return fail(TSPH_ERR_ARG, "h and kap must be positive");
    HostSetup hs;
    hs.h = c->h;
    hs.kap = c->kap;
    hs.x0 = d->x_0;
    hs.xm = d->x_m;
    hs.y0 = d->y_0;
    hs.ym = d->y_m;
    int rc = make_grid(hs);
    if (rc) return rc;
    *ncx = hs.ncx;
    *ncy = hs.ncy;
    if (bx) std::memcpy(bx, hs.bx.data(), 8 * hs.bx.size());
    if (by) std::memcpy(by, hs.by.data(), 8 * hs.by.size());
    return TSPH_OK;
}

// Divide_To_Cells, src/SPH_find_pairs.h:5-42
int tsph_divide_to_cells(tsph_system *s) {
    NEED(s);
    int rc = make_grid(s->hs);
    if (rc) return rc;
    s->divided = true;
    s->stale_engine = true;
    return TSPH_OK;
}

int tsph_clear_cells(tsph_system *s) {
    NEED(s);
    if (s->eng && !s->stale_engine) s->eng->invalidate_cells();
    return TSPH_OK;
}

int tsph_particle_to_cell(tsph_system *s) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->particle_to_cell(err_));
    return TSPH_OK;
}

int tsph_get_cells(tsph_system *s, int32_t *cell_start, int32_t *cell_list) {
    NEED(s);
    if (!cell_start || !cell_list) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    RUN(s->eng->get_cells(cell_start, cell_list, err_));
    return TSPH_OK;
}

int tsph_pair_digest(tsph_system *s, int32_t *count, int64_t *sum, int32_t *xor_) {
    NEED(s);
    if (!count || !sum || !xor_) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    RUN(s->eng->pair_digest(count, sum, xor_, err_));
    return TSPH_OK;
}

int tsph_density_to_pressure(tsph_system *s) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->density_to_pressure(err_));
    return TSPH_OK;
}

int tsph_mdbc_density(tsph_system *s) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->mdbc_density(err_));
    return TSPH_OK;
}

int tsph_add_buffer_zone(tsph_system *s, double x0, double xm, double y0, double ym, int nbl,
                         double vx, double vy, double ox, double oy, int btype) {
    NEED(s);
    if (!((ox != 0) ^ (oy != 0)) || btype < 2 || btype > 255)
        return fail(TSPH_ERR_ARG, "zone orientation must be along x or y, btype in [2, 255]");
    // BufferZone constructor, src/SPH_inlet_outlet_data.h
    double bl = std::fabs(xm - x0), bh = std::fabs(ym - y0);
    if (oy != 0) {
        bl = std::fabs(ym - y0);
        bh = std::fabs(xm - x0);
    }
    const double z[12] = {ox, oy, x0, y0, xm, ym, (double)nbl, bl, bh, (double)btype, vx, vy};
    s->hs.zones.insert(s->hs.zones.end(), z, z + 12);
    s->stale_engine = true;
    return TSPH_OK;
}

int tsph_set_cases(tsph_system *s, int ncases, const double *x_range, const double *gravity,
                   const double *removal) {
    NEED(s);
    if (ncases < 0 || (ncases > 0 && (!x_range || !gravity || !removal)))
        return fail(TSPH_ERR_ARG, "tsph_set_cases: ncases >= 0 and the three arrays");
    if (s->precision == TSPH_PREC_FP64)
        return fail(TSPH_ERR_UNSUPPORTED, "tsph_set_cases: FP32 build only");
    for (int k = 0; k < ncases; k++)
        if (!(x_range[2 * k] < x_range[2 * k + 1]) || !(removal[4 * k] < removal[4 * k + 1]) ||
            !(removal[4 * k + 2] < removal[4 * k + 3]))
            return fail(TSPH_ERR_ARG, "tsph_set_cases: empty range of case " + std::to_string(k));
    {  // cases do not share columns: their x ranges are disjoint
        std::vector<std::pair<double, double>> xr((size_t)ncases);
        for (int k = 0; k < ncases; k++) xr[k] = {x_range[2 * k], x_range[2 * k + 1]};
        std::sort(xr.begin(), xr.end());
        for (int k = 1; k < ncases; k++)
            if (xr[k].first < xr[k - 1].second)
                return fail(TSPH_ERR_ARG, "tsph_set_cases: the x ranges of two cases overlap");
    }
    s->hs.case_x.assign(x_range, x_range + 2 * (size_t)ncases);
    s->hs.case_g.assign(gravity, gravity + (size_t)ncases);
    s->hs.case_box.assign(removal, removal + 4 * (size_t)ncases);
    s->stale_engine = true;
    return TSPH_OK;
}

int tsph_set_zone_capacity(tsph_system *s, int extra_rows, int extra_ids) {
    NEED(s);
    if (extra_rows < 0 || extra_ids < 0) return fail(TSPH_ERR_ARG, "capacities must be >= 0");
    s->hs.extra_rows = extra_rows;
    s->hs.extra_ids = extra_ids;
    s->stale_engine = true;
    return TSPH_OK;
}

int tsph_bz_inlet(tsph_system *s, int zone, double dt) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->bz_inlet(zone, dt, err_));
    return TSPH_OK;
}

int tsph_bz_outlet(tsph_system *s, int zone, double dt) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->bz_outlet(zone, dt, err_));
    return TSPH_OK;
}

int tsph_bt_density(tsph_system *s) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->bt_density(err_));
    return TSPH_OK;
}

int tsph_compute_forces(tsph_system *s, int wall_model) {
    NEED(s);
    if (wall_model != TSPH_WALL_MDBC && wall_model != TSPH_WALL_DBC && wall_model != TSPH_WALL_BT)
        return fail(TSPH_ERR_ARG, "wall_model must be TSPH_WALL_MDBC, TSPH_WALL_DBC or TSPH_WALL_BT");
    ENGINE(s);
    RUN(s->eng->compute_forces(wall_model, err_));
    return TSPH_OK;
}

int tsph_symplectic_predictor(tsph_system *s, double dt) {
    NEED(s);
    if (!std::isfinite(dt)) return fail(TSPH_ERR_ARG, "dt must be finite");
    ENGINE(s);
    RUN(s->eng->predictor(dt, err_));
    return TSPH_OK;
}

int tsph_symplectic_corrector(tsph_system *s, double dt) {
    NEED(s);
    if (!std::isfinite(dt)) return fail(TSPH_ERR_ARG, "dt must be finite");
    ENGINE(s);
    RUN(s->eng->corrector(dt, err_));
    return TSPH_OK;
}

int tsph_remove_out_of_domain(tsph_system *s, int *removed) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->remove_out_of_domain(removed, err_));
    return TSPH_OK;
}

int tsph_step(tsph_system *s, int wall_model, double dt, int nsteps) {
    NEED(s);
    if (wall_model != TSPH_WALL_MDBC && wall_model != TSPH_WALL_DBC && wall_model != TSPH_WALL_BT)
        return fail(TSPH_ERR_ARG, "wall_model must be TSPH_WALL_MDBC, TSPH_WALL_DBC or TSPH_WALL_BT");
    if (!std::isfinite(dt) || nsteps < 0) return fail(TSPH_ERR_ARG, "bad dt or nsteps");
    ENGINE(s);
    if (nsteps == 0) return TSPH_OK;
    RUN(s->eng->step(wall_model, dt, nsteps, err_));
    return TSPH_OK;
}

int tsph_download(tsph_system *s, int fields, const tsph_host_state *out) {
    NEED(s);
    if (!out) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    RUN(s->eng->download(fields, out->r, out->v, out->a, out->rho, out->drho, out->p, out->index,
                         (fields & TSPH_F_TYPE) ? out->type : nullptr, err_));
    if ((fields & TSPH_F_TYPE) && out->type && s->hs.zones.empty()) {
        // types from the host list, in the reference's order of live particles
        // (systems with buffer zones read them from the device above)
        std::vector<int32_t> idx;
        int np = 0;
        RUN(s->eng->np_live(&np, err_));
        idx.resize(np);
        RUN(s->eng->download(TSPH_F_INDEX, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                             idx.data(), nullptr, err_));
        for (int k = 0; k < np; k++) out->type[k] = s->hs.type[idx[k]];
    }
    return TSPH_OK;
}

int tsph_download_async(tsph_system *s, int fields, const tsph_host_state *out) {
    NEED(s);
    if (!out) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    RUN(s->eng->download_async(fields, out->r, out->v, out->a, out->rho, out->drho, out->p,
                               err_));
    return TSPH_OK;
}

int tsph_upload_async(tsph_system *s, int fields, const tsph_host_state *in) {
    NEED(s);
    if (!in) return fail(TSPH_ERR_ARG, "null input");
    ENGINE(s);
    RUN(s->eng->upload_async(fields, in->r, in->v, in->a, in->rho, in->drho, in->p, err_));
    return TSPH_OK;
}

int tsph_download_wait(tsph_system *s) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->download_wait(err_));
    return TSPH_OK;
}

int tsph_upload(tsph_system *s, int fields, const tsph_host_state *in) {
    NEED(s);
    if (!in) return fail(TSPH_ERR_ARG, "null input");
    if (fields & (TSPH_F_INDEX | TSPH_F_TYPE))
        return fail(TSPH_ERR_ARG, "index and type are not uploadable");
    ENGINE(s);
    RUN(s->eng->upload(fields, in->r, in->v, in->a, in->rho, in->drho, in->p, err_));
    return TSPH_OK;
}

int tsph_sync(tsph_system *s) {
    NEED(s);
    if (!s->eng) return TSPH_OK;
    RUN(s->eng->sync(err_));
    return TSPH_OK;
}

int tsph_kernel_launches(tsph_system *s, long long *count, int reset) {
    NEED(s);
    if (!count) return fail(TSPH_ERR_ARG, "null count");
    if (!s->eng) {
        *count = 0;
        return TSPH_OK;
    }
    RUN(s->eng->kernel_launches(count, reset, err_));
    return TSPH_OK;
}

int tsph_health(tsph_system *s, uint32_t *flags, int clear) {
    NEED(s);
    if (!flags) return fail(TSPH_ERR_ARG, "null flags");
    if (!s->eng || s->stale_engine) {
        *flags = 0;
        return TSPH_OK;
    }
    RUN(s->eng->health(flags, clear, err_));
    return TSPH_OK;
}

int tsph_fluid_totals(tsph_system *s, double out[4]) {
    NEED(s);
    if (!out) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    RUN(s->eng->totals(out, err_));
    return TSPH_OK;
}

int tsph_water_level(tsph_system *s, int n, const double *x, const double *y0,
                     const int32_t *inverse, double *out) {
    NEED(s);
    if (n < 0 || (n > 0 && (!x || !y0 || !out))) return fail(TSPH_ERR_ARG, "bad arguments");
    if (n == 0) return TSPH_OK;
    ENGINE(s);
    RUN(s->eng->water_level(n, x, y0, inverse, out, err_));
    return TSPH_OK;
}

int tsph_point_fields(tsph_system *s, int n, const double *xy, double *out) {
    NEED(s);
    if (n < 0 || (n > 0 && (!xy || !out))) return fail(TSPH_ERR_ARG, "bad arguments");
    if (n == 0) return TSPH_OK;
    ENGINE(s);
    RUN(s->eng->point_fields(n, xy, out, err_));
    return TSPH_OK;
}

int tsph_water_front(tsph_system *s, double y_max, double *x_front) {
    NEED(s);
    if (!x_front) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    RUN(s->eng->water_front(y_max, x_front, err_));
    return TSPH_OK;
}

int tsph_export_graph(tsph_system *s, int k_slots, int capacity, void *pos, void *vel,
                      float *srho, float *wall, int32_t *id, int32_t *deg, int32_t *nbr,
                      void *acc, float *rate, int32_t *n_nodes, int32_t *n_wall) {
    NEED(s);
    if (k_slots < 1 || capacity < 0 || !pos || !vel || !srho || !wall || !id || !deg || !nbr ||
        !n_nodes || !n_wall)
        return fail(TSPH_ERR_ARG, "bad arguments");
    ENGINE(s);
    int n = 0, nw = 0;
    RUN(s->eng->export_graph(k_slots, capacity, static_cast<double2 *>(pos),
                             static_cast<float2 *>(vel), srho, wall, id, deg, nbr,
                             static_cast<float2 *>(acc), rate, &n, &nw, err_));
    *n_nodes = n;
    *n_wall = nw;
    return TSPH_OK;
}

int tsph_apply_update(tsph_system *s, const float *y, double u_scale, double s_scale,
                      double k_dt, int flags, int phase) {
    NEED(s);
    if (!y) return fail(TSPH_ERR_ARG, "null update");
    if (phase < 0 || phase > 2) return fail(TSPH_ERR_ARG, "phase must be 0, 1 or 2");
    ENGINE(s);
    RUN(s->eng->apply_update(y, u_scale, s_scale, k_dt, (flags & TSPH_UPDATE_RATES) != 0,
                             (flags & TSPH_UPDATE_ZERO_MOMENTUM) != 0, phase, err_));
    return TSPH_OK;
}

int tsph_window_check(tsph_system *s, double k_dt, double out[5]) {
    NEED(s);
    if (!out) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    RUN(s->eng->window_check(k_dt, out, err_));
    return TSPH_OK;
}

int tsph_get_stream(tsph_system *s, void **stream) {
    NEED(s);
    if (!stream) return fail(TSPH_ERR_ARG, "null output");
    ENGINE(s);
    *stream = s->eng->stream();
    return TSPH_OK;
}

int tsph_state_save(tsph_system *s) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->state_save(err_));
    return TSPH_OK;
}

int tsph_state_restore(tsph_system *s) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->state_restore(err_));
    return TSPH_OK;
}

int tsph_autotune(tsph_system *s, int32_t *shape, double us[TSPH_N_TILE_SHAPES]) {
    NEED(s);
    ENGINE(s);
    int c = 0;
    RUN(s->eng->autotune(&c, us, err_));
    if (shape) *shape = c;
    return TSPH_OK;
}

int tsph_set_tile_shape(tsph_system *s, int shape) {
    NEED(s);
    ENGINE(s);
    RUN(s->eng->set_tile_shape(shape, err_));
    return TSPH_OK;
}

int tsph_get_tile_shape(tsph_system *s, int32_t *shape) {
    NEED(s);
    ENGINE(s);
    if (!shape) return fail(TSPH_ERR_ARG, "tsph_get_tile_shape: shape is NULL");
    *shape = s->eng->tile_shape();
    return TSPH_OK;
}

int tsph_set_profiling(tsph_system *s, int on) {
    NEED(s);
    s->profiling = on != 0;
    if (s->eng) s->eng->set_profiling(s->profiling);
    return TSPH_OK;
}

int tsph_get_profile(tsph_system *s, tsph_profile_t *out, int reset) {
    NEED(s);
    if (!out) return fail(TSPH_ERR_ARG, "null output");
    std::memset(out, 0, sizeof(*out));
    if (!s->eng) return TSPH_OK;
    tsph::Profile p = s->eng->profile(reset != 0);
    out->pair_us = p.us[tsph::CAT_PAIR];
    out->pair_launches = p.launches[tsph::CAT_PAIR];
    out->sort_us = p.us[tsph::CAT_SORT];
    out->sort_launches = p.launches[tsph::CAT_SORT];
    out->mdbc_us = p.us[tsph::CAT_MDBC];
    out->mdbc_launches = p.launches[tsph::CAT_MDBC];
    out->other_us = p.us[tsph::CAT_OTHER];
    out->other_launches = p.launches[tsph::CAT_OTHER];
    return TSPH_OK;
}

}  // extern "C"
