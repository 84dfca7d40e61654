// tsph_engine.cuh -- Engine<T>: device buffers, kernel sequencing, CUDA-graph
// replay of the fused step.  Included once per precision.
#pragma once

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <utility>
#include <vector>

#include "tsph_engine.h"
#include "tsph_kernels.cuh"
#include "tsph_pairs_tiled.cuh"
#include "tsph_pairs_rec.cuh"
#include "tsph_probes.cuh"
#include "tsph_graph.cuh"
#include "tsph_zones.cuh"
#include "tsph_grid_host.h"

namespace tsph {

#define TSPH_CK(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) {                                                   \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);              \
            return 2; /* TSPH_ERR_CUDA */                                          \
        }                                                                          \
    } while (0)

static inline int blocks_for(long long n, int b = kBlock) {
    return (int)std::max<long long>(1, (n + b - 1) / b);
}

template <typename T> class Engine final : public EngineBase {
    typedef typename V2<T>::t T2;

    // ---- sizes
    int nf_ = 0, nw_ = 0, ntot_ = 0;  // fluid rows (capacity), walls, particle indices in use
    int id_cap_ = 0;                  // capacity of the index space (grows with inlets)
    // open boundaries (buffer zones)
    bool zones_on_ = false;
    std::vector<ZoneDev> zones_;
    uint32_t *zlist_ = nullptr, *zcount_ = nullptr;
    int zlist_cap_ = 0;
    uint8_t *zlive_ = nullptr, *zcand_ = nullptr;
    // the fused step's RemoveParticlesOutOfDomain: erase candidates and the
    // indices removed so far
    uint8_t *rm_cand_ = nullptr, *dead_ = nullptr;
    uint32_t *rm_list_ = nullptr, *rm_count_ = nullptr;
    int ncells_ = 0;
    Grid grid_{};
    Phys<T> P_{};
    Box box_{};
    cudaStream_t st_ = nullptr;
    bool own_stream_ = false;
    bool cells_ = false;
    double m64_ = 0, dp64_ = 0;
    // probe scratch (grown on demand)
    double *pr_d_ = nullptr;
    size_t pr_cap_ = 0;

    // ---- device memory (one arena per kind; freed in the destructor)
    std::vector<void *> allocs_;
    FluidState<T> F_{}, Fs_{};  // current sorted state, predicted sorted state
    OldState<T> O_{};
    double2 *Br_ = nullptr;
    T2 *Bv_ = nullptr;
    T *Brho_ = nullptr;
    uint32_t *keyB_ = nullptr, *slotB_ = nullptr, *tmp_id_ = nullptr, *tmp_src_ = nullptr,
             *perm_ = nullptr;
    uint32_t *counts_ = nullptr, *fstart_ = nullptr, *wstart_ = nullptr, *tile_sums_ = nullptr;
    long long *tmp_y_ = nullptr;
    uint32_t *health_ = nullptr, *removed_ = nullptr;
    uint32_t *rebuild_ = nullptr;  // set when the fused step must re-bin after the predictor
    bool exported_ = false;        // the sorted order is that of the last export_graph
    WindowRef wref_{};             // start-of-window terms of the surrogate's check
    double *wout_ = nullptr;       // its reductions
    double *ymean_ = nullptr;      // sums of the update's (y0, y1) over the fluid, and the count
    FluidState<T> Fsv_{};          // the saved state (tsph_state_save)
    T *wsv_ = nullptr;             // saved wall rho, drho, p, rho_o (4 nw)
    uint32_t *fstart_sv_ = nullptr;
    bool saved_ = false, saved_cells_ = false, saved_kept_ = false;
    bool kicked_ = false;          // a kick (apply_update phase 1) awaits its drift
    bool capturing_ = false;       // enqueue_step is being captured into a graph
    cudaStream_t st2_ = nullptr;   // side stream: captures the conditional re-binning body
    float skin_ = 0.f;             // per-axis move allowed without re-binning (FP32 fused step)
    WallState<T> W_{};
    Staging S_{};
    // asynchronous download: its own staging set, copy stream and events
    Staging D_{};
    cudaStream_t cs_ = nullptr;
    cudaEvent_t ev_x_ = nullptr, ev_d_ = nullptr;
    bool d_pending_ = false;
    // staged upload: host-to-device copies into S_ on their own stream,
    // applied by the next particle_to_cell
    cudaStream_t cu_ = nullptr;
    cudaEvent_t ev_up_ = nullptr, ev_imp_ = nullptr;
    bool up_pending_ = false;
    int up_mask_ = 0;
    double *dtot_ = nullptr;
    long long *bx_ = nullptr, *by_ = nullptr;
    double *ox_ = nullptr, *oy_ = nullptr;
    int32_t *dig_count_ = nullptr, *dig_xor_ = nullptr;
    long long *dig_sum_ = nullptr;

    // ---- graphs keyed by (model, dt bits)
    std::map<std::pair<int, long long>, cudaGraphExec_t> graphs_;
    // kernel launches: eager ones counted as they are made; a graph's kernels
    // counted at capture (outside / inside each conditional body: 1 the
    // re-binning after the predictor, 2 the sort after the corrector, 3 the
    // in-order copy instead of it), its launches then add the outside ones and
    // the bodies' executions (counted on the device in body_runs_) add theirs
    long long launched_ = 0;
    int cap_main_ = 0, cap_body_[4] = {0, 0, 0, 0}, body_kernels_[4] = {0, 0, 0, 0};
    int body_ = 0;  // the conditional body being captured (0: none)
    uint32_t *body_runs_ = nullptr;  // [1..3]: executions of each body
    std::map<std::pair<int, long long>, int> graph_kernels_;

    // ---- profiling
    bool prof_ = false;
    // programmatic dependent launch of the engine's kernels (TSPH_PDL=0 turns
    // it off, e.g. to compare)
    bool pdl_ = true;
    struct Mark {
        int cat;
        cudaEvent_t a, b;
    };
    std::vector<Mark> marks_;
    std::vector<cudaEvent_t> ev_pool_;
    Profile acc_{};

    template <typename P> int alloc(P **p, size_t count, std::string &err) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(P));
        if (e != cudaSuccess) {
            err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
            return 4;
        }
        allocs_.push_back(q);
        *p = static_cast<P *>(q);
        return 0;
    }

    cudaEvent_t ev() {
        if (ev_pool_.empty()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            return e;
        }
        cudaEvent_t e = ev_pool_.back();
        ev_pool_.pop_back();
        return e;
    }

    // The state's pressure array after tsph_step.  The step's own passes form
    // p = EOS(rho) inside their pair records and never read the array, so a
    // step only marks it out of date; every other entry point first runs the
    // EOS over the state (TSPH_FRESH_P), so what any call sees or replaces is
    // the state the reference's step leaves (p = EOS(rho), its step body
    // :110-111), without an EOS launch per step of a time loop.
    bool p_stale_ = false;
    static constexpr int kFieldP = 1 << 5;  // the pressure's bit in a field mask (TSPH_F_P)
    int fresh_p(std::string &err) {
        if (!p_stale_) return 0;
        const int rc = launch(CAT_OTHER, k_eos<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                              (const uint32_t *)fstart_, ncells_, W_, nw_, P_, health_);
        if (rc == 0) p_stale_ = false;
        return rc;
    }
#define TSPH_FRESH_P(err)                     \
    do {                                      \
        const int rc_p_ = fresh_p(err);       \
        if (rc_p_) return rc_p_;              \
    } while (0)

    // launch with optional event bracketing for the profile.  Every kernel
    // launched here begins with pdl_enter(), so it may be launched with
    // programmatic stream serialisation: its launch overlaps the previous
    // kernel's tail, its first instruction waits for that kernel.
    template <typename K, typename... A>
    int launch(int cat, K kern, int grid, int block, std::string &err, A... args) {
        cudaEvent_t a = nullptr, b = nullptr;
        if (prof_) {
            a = ev();
            b = ev();
            cudaEventRecord(a, st_);
        }
        if (!capturing_) launched_++;
        else if (body_) cap_body_[body_]++;
        else cap_main_++;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3((unsigned)block);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st_;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = pdl_ ? 1 : 0;
        cudaError_t e = cudaLaunchKernelEx(&cfg, kern, args...);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            err = std::string("kernel launch: ") + cudaGetErrorString(e);
            return 2;
        }
        if (prof_) {
            cudaEventRecord(b, st_);
            marks_.push_back({cat, a, b});
        }
        return 0;
    }

    int collect_profile(std::string &err) {
        if (!prof_ || marks_.empty()) return 0;
        TSPH_CK(cudaStreamSynchronize(st_));
        for (auto &m : marks_) {
            float ms = 0;
            cudaEventElapsedTime(&ms, m.a, m.b);
            acc_.us[m.cat] += 1000.0 * ms;
            acc_.launches[m.cat] += 1;
            ev_pool_.push_back(m.a);
            ev_pool_.push_back(m.b);
        }
        marks_.clear();
        return 0;
    }

    Nbr<T> nbr_fluid(const FluidState<T> &X, bool stored_p) const {
        return Nbr<T>{X.r, X.loc, X.v, X.rho, stored_p ? X.p : nullptr, nullptr, X.type};
    }
    // walls have v = 0: the pair loop reads a zero velocity array
    T2 *wall_zero_v_ = nullptr;

    Nbr<T> nbr_walls(bool stored_p) const {
        return Nbr<T>{W_.r, W_.loc, wall_zero_v_, W_.rho, stored_p ? W_.p : nullptr};
    }
    // boundary-integral walls: the per-wall vector of tsph_add_particles is the normal
    Nbr<T> nbr_walls_bt(bool stored_p) const {
        return Nbr<T>{W_.r, W_.loc, wall_zero_v_, W_.rho, stored_p ? W_.p : nullptr, W_.gnr};
    }
    int wall_model_ = 0;  // wall model of the pass being enqueued (2: boundary integral)

    int do_bt_density(std::string &err) {
        if (nw_ == 0) return 0;
        return launch(CAT_MDBC, k_bt_density<T>, blocks_for(nw_), kBlock, err, W_, nw_,
                      (const uint32_t *)fstart_, nbr_fluid(F_, false), grid_, P_);
    }

    // scan counts[0..ncells] -> fstart[0..ncells+1]; leaves counts zeroed
    int scan(std::string &err, const uint32_t *gate = nullptr) {
        const int n = ncells_ + 1;
        const int ntiles = (n + kScanTile - 1) / kScanTile;
        int rc;
        if ((rc = launch(CAT_SORT, k_scan_tiles_clear, ntiles, kScanThreads, err, counts_, fstart_,
                         tile_sums_, n, gate)))
            return rc;
        return launch(CAT_SORT, k_scan_add_tiles, blocks_for(n), kBlock, err, fstart_,
                      (const uint32_t *)tile_sums_, ntiles, n, gate);
    }

    // after keys/slots are in keyB_/slotB_ and counts_ is filled:
    // scan, stable placement, rank + scatter of the source arrays into D (+ old state)
    int sort_finish(const double2 *sr, const T2 *sv, const T *srho, const uint32_t *sid,
                    const T2 *sa, const T *sdrho, const T *sp, FluidState<T> D,
                    const double2 *or2, const T2 *ov2, const T *orho2, OldState<T> Od,
                    std::string &err, const uint32_t *gate = nullptr,
                    const uint8_t *stype = nullptr, uint32_t *runs = nullptr) {
        int rc;
        if ((rc = scan(err, gate))) return rc;
        const int *ntot = reinterpret_cast<const int *>(fstart_ + ncells_ + 1);
        const int nb = blocks_for(nf_);
        // FP32 build: cells ordered by (y, index); FP64 build: by index
        constexpr bool by_y = std::is_same<T, float>::value;
        if ((rc = launch(CAT_SORT, k_place, nb, kBlock, err, (const uint32_t *)keyB_,
                         (const uint32_t *)slotB_, sid, ntot, (const uint32_t *)fstart_, tmp_id_,
                         tmp_src_, by_y ? sr : (const double2 *)nullptr, tmp_y_, gate)))
            return rc;
        return launch(CAT_SORT, k_rank_scatter<T>, nb, kBlock, err, (const uint32_t *)keyB_, ntot,
                      (const uint32_t *)fstart_, (const uint32_t *)tmp_id_,
                      (const uint32_t *)tmp_src_,
                      by_y ? (const long long *)tmp_y_ : (const long long *)nullptr, grid_, sr, sv,
                      srho, sid, sa, sdrho, sp, D, or2, ov2, orho2, Od, gate,
                      D.type ? stype : (const uint8_t *)nullptr, lbin_, gen_, runs);
    }

    // the histogram is zero between sorts (the scan clears it)
    int zero_counts(std::string &err) {
        (void)err;
        return 0;
    }

    int do_mdbc(std::string &err) {
        if (nw_ == 0) return 0;
        if constexpr (std::is_same<T, float>::value) {
            const int lanes = mdbc_lanes(nw_, sm_count_);
            return launch(CAT_MDBC, lanes == kMdbcLanes ? k_mdbc_f32<kMdbcLanes>
                                                        : k_mdbc_f32<kMdbcLanesMany>,
                          blocks_for((long long)nw_ * lanes), kBlock, err, W_, nw_,
                          (const uint32_t *)fstart_, F_, grid_, P_);
        } else
            return launch(CAT_MDBC, k_mdbc<T>, blocks_for((long long)nw_ * 32), kBlock, err, W_,
                          nw_, (const uint32_t *)fstart_, nbr_fluid(F_, false), grid_, P_);
    }

    TileConst K_{}, Kskin_{};
    int tile_shape_ = -1;  // 0 TileWide, 1 TileDeep, 2 pair records; -1: not tuned yet
    // pair records (tile shape 2): of F_, of Fs_, of the walls
    PairRec rec_f_{}, rec_s_{}, rec_w_{};
    WinRec *rec_table_ = nullptr;  // windows of each chunk of 128 targets
    int *rec_nwin_ = nullptr;
    TileConst Krec_{}, Krec_build_{};  // pair terms / list building (radius 2h + 2 sigma)
    bool rec_setup_ = false;
    int tiled_best_ = 0;  // the faster of shapes 0 and 1 (per-function calls with shape 2)
    // cells kept over several steps (fused step with shape 2)
    float2 *lbin_ = nullptr;      // cell-relative positions at the last binning (F_ order)
    uint16_t *rec_list_ = nullptr;
    uint8_t *rec_cnt_ = nullptr;
    uint32_t *gen_ = nullptr;     // {sorts, sort the lists were built after, -, CTAs done}
    uint32_t *need_sort_ = nullptr;
    uint32_t *pc_gate_ = nullptr;  // set when an applied upload cannot keep the cells
    int sm_count_ = 152;           // the device's SMs (grid shapes)
    bool binned_ = false;          // a binning has formed lbin_ and the lists
    float sig2_ = 0.f;
    bool cells_kept_ = false;     // F_ moved since its binning (within sigma)
    long long rec_passes_ = 0;    // kept-list pair passes run (host count)
    long long rec_passes_sv_ = -1;
    float2 *lbin_sv_ = nullptr;   // binning positions and list counters at state_save
    uint32_t *gen_sv_ = nullptr;
    // cases packed into one system (tsph_set_cases): the case of each grid
    // column and each case's gravity-dependent constants and removal box
    int32_t *col_case_ = nullptr;
    CaseConst *cases_ = nullptr;
    bool cases_on_ = false;

    // The case table of HostSetup on the device.  A column belongs to the case
    // whose x range holds its centre (a column between ranges, to the nearest
    // case); per case, gravity, the Fourtakas coefficients that follow from it
    // (as make_tile_const forms them) and the removal thresholds as ordered
    // bits.
    int setup_cases(const HostSetup &hs, std::string &err) {
        const int nc = (int)hs.case_g.size();
        if ((int)hs.case_x.size() != 2 * nc || (int)hs.case_box.size() != 4 * nc) {
            err = "case table: 2 x-range values, 1 gravity and 4 thresholds per case";
            return 1;
        }
        std::vector<int32_t> cc(hs.ncx, -1);
        for (int k = 0; k < nc; k++) {
            const double lo = hs.case_x[2 * k], hi = hs.case_x[2 * k + 1];
            // first column whose centre is at or above lo
            int cx = (int)(std::lower_bound(hs.ox.begin(), hs.ox.end(), lo - 0.5 * hs.kh) -
                           hs.ox.begin());
            for (; cx < hs.ncx && hs.ox[cx] + 0.5 * hs.kh < hi; cx++)
                if (hs.ox[cx] + 0.5 * hs.kh >= lo) cc[cx] = k;
        }
        int last = -1;
        std::vector<int> dist(hs.ncx, 1 << 30);
        for (int cx = 0; cx < hs.ncx; cx++) {  // nearest assigned column on the left
            if (cc[cx] >= 0) last = cx;
            else if (last >= 0) dist[cx] = cx - last;
        }
        std::vector<int32_t> out = cc;
        for (int cx = 0; cx < hs.ncx; cx++)
            if (cc[cx] < 0 && dist[cx] < (1 << 30)) out[cx] = cc[cx - dist[cx]];
        last = -1;
        for (int cx = hs.ncx - 1; cx >= 0; cx--) {  // or on the right, when nearer
            if (cc[cx] >= 0) {
                last = cx;
            } else if (last >= 0 && last - cx < dist[cx]) {
                out[cx] = cc[last];
            }
        }
        for (int cx = 0; cx < hs.ncx; cx++)
            if (out[cx] < 0) {
                err = "case table: no case covers the grid";
                return 1;
            }
        std::vector<CaseConst> C(nc);
        for (int k = 0; k < nc; k++) {
            const double g = hs.case_g[k];
            const double xg = 7.0 * g / (hs.cs * hs.cs);
            C[k].g = (float)g;
            C[k].c1 = (float)(hs.rho0 * xg / 7.0);
            C[k].c2 = (float)(-hs.rho0 * 3.0 / 49.0 * xg * xg);
            C[k].pad = 0.f;
            const double *b = &hs.case_box[4 * k];
            C[k].box = BoxBits{ordered_bits_fold0(b[0]), ordered_bits_fold0(b[1]),
                               ordered_bits_fold0(b[2]), ordered_bits_fold0(b[3])};
        }
        int rc;
        if ((rc = alloc(&col_case_, hs.ncx, err)) || (rc = alloc(&cases_, nc, err))) return rc;
        TSPH_CK(cudaMemcpy(col_case_, out.data(), 4 * (size_t)hs.ncx, cudaMemcpyHostToDevice));
        TSPH_CK(cudaMemcpy(cases_, C.data(), sizeof(CaseConst) * (size_t)nc,
                           cudaMemcpyHostToDevice));
        cases_on_ = true;
        tile_shape_ = 2;  // the pair-record kernel is the one that reads the table
        return 0;
    }

  public:
    // time every pair-kernel variant on the current particles (forces pass,
    // a and drho saved and restored): a warm-up and 20 timed launches each,
    // the median kept; the fastest wins.  FP32 build only.
    static constexpr int kShapes = 3;
    int autotune(int *choice, double *us, std::string &err) override {
        TSPH_FRESH_P(err);
        if (cases_on_) {  // packed cases: the pair-record kernel only
            if (choice) *choice = 2;
            if (us)
                for (int k = 0; k < kShapes; k++) us[k] = 0;
            return 0;
        }
        // the FP64 build, boundary-integral walls and buffer zones use the
        // per-particle pair kernel: nothing to choose
        if (!std::is_same<T, float>::value || wall_model_ == 2 || zones_on_) {
            tile_shape_ = 0;
            if (choice) *choice = 0;
            if (us)
                for (int k = 0; k < kShapes; k++) us[k] = 0;
            return 0;
        } else {
            if (!cells_ok()) {
                err = "cell lists are stale: call tsph_particle_to_cell first";
                return 3;
            }
            int rc0;
            if ((rc0 = ensure_exact_cells(err))) return rc0;
            const bool prof = prof_;
            prof_ = false;
            TSPH_CK(cudaMemcpyAsync(Bv_, F_.a, sizeof(T2) * (size_t)nf_, cudaMemcpyDeviceToDevice, st_));
            TSPH_CK(cudaMemcpyAsync(Brho_, F_.drho, sizeof(T) * (size_t)nf_, cudaMemcpyDeviceToDevice, st_));
            constexpr int kReps = 20;
            std::vector<cudaEvent_t> evs(kReps + 1);
            for (auto &e : evs) e = ev();
            double med[kShapes] = {0, 0, 0};
            int rc = 0;
            for (int shape = 0; shape < kShapes && !rc; shape++) {
                tile_shape_ = shape;
                tiled_best_ = shape == 2 ? tiled_best_ : shape;
                // shape 2 as the fused step runs it: the first pass builds the
                // lists (its state is as binned), the timed ones sum them
                auto pass = [&]() {
                    return shape == 2 ? fluid_pairs_rec<MODE_FORCES>(F_, T(0), PairOut{}, err)
                                      : fluid_pairs<MODE_FORCES>(F_, false, T(0), PairOut{}, err);
                };
                rc = pass();  // warm
                cudaEventRecord(evs[0], st_);
                for (int rep = 0; rep < kReps && !rc; rep++) {
                    rc = pass();
                    cudaEventRecord(evs[rep + 1], st_);
                }
                if (rc) break;
                cudaEventSynchronize(evs[kReps]);
                std::vector<float> t(kReps);
                for (int rep = 0; rep < kReps; rep++)
                    cudaEventElapsedTime(&t[rep], evs[rep], evs[rep + 1]);
                std::sort(t.begin(), t.end());
                med[shape] = 0.5 * (t[kReps / 2 - 1] + t[kReps / 2]);
                if (shape == 1) tiled_best_ = med[1] < med[0] ? 1 : 0;
            }
            for (auto &e : evs) ev_pool_.push_back(e);
            prof_ = prof;
            if (rc) return rc;
            TSPH_CK(cudaMemcpyAsync(F_.a, Bv_, sizeof(T2) * (size_t)nf_, cudaMemcpyDeviceToDevice, st_));
            TSPH_CK(cudaMemcpyAsync(F_.drho, Brho_, sizeof(T) * (size_t)nf_, cudaMemcpyDeviceToDevice, st_));
            TSPH_CK(cudaStreamSynchronize(st_));
            int best = 0;
            for (int k = 1; k < kShapes; k++)
                if (med[k] < med[best]) best = k;
            tile_shape_ = best;
            // graphs captured with another variant are stale
            for (auto &g : graphs_) cudaGraphExecDestroy(g.second);
            graphs_.clear();
            if (choice) *choice = tile_shape_;
            if (us)
                for (int k = 0; k < kShapes; k++) us[k] = 1000.0 * med[k];
            return 0;
        }
    }

    int tile_shape() const override { return tile_shape_; }

    void *stream() const override { return st_; }

    int export_graph(int K, int cap, double2 *pos, float2 *vel, float *srho, float *wall,
                     int32_t *id, int32_t *deg, int32_t *nbr, float2 *acc, float *rate,
                     int *n_nodes, int *n_wall, std::string &err) override {
        TSPH_FRESH_P(err);
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        uint32_t nl = 0;
        TSPH_CK(cudaMemcpyAsync(&nl, fstart_ + ncells_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        const int n = nw_ + (int)nl;
        *n_nodes = n;
        *n_wall = nw_;
        if (n > cap) {
            err = "graph capacity " + std::to_string(cap) + " < " + std::to_string(n) + " nodes";
            return 1;
        }
        int rc;
        TSPH_CK(cudaMemsetAsync(removed_, 0, 4, st_));
        if ((rc = launch(CAT_OTHER, k_graph_export<T>, blocks_for(n), kBlock, err, F_,
                         (const uint32_t *)fstart_, (const uint32_t *)wstart_, W_, nw_, grid_,
                         P_.rho0, (float)(4.0 * P_.hd * P_.hd), K, pos, vel, srho, wall, id, deg,
                         nbr, acc, rate, removed_)))
            return rc;
        uint32_t ovf = 0;
        TSPH_CK(cudaMemcpyAsync(&ovf, removed_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaMemsetAsync(removed_, 0, 4, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        if (ovf) {
            err = "a node has more than " + std::to_string(K) + " neighbours";
            return 8;
        }
        exported_ = true;
        kicked_ = false;
        return collect_profile(err);
    }

    int apply_update(const float *y, double su, double ss, double kdt, bool add_rates,
                     bool zero_momentum, int phase, std::string &err) override {
        TSPH_FRESH_P(err);
        if (!exported_ || !cells_ok()) {
            err = "apply_update needs the order of the last export_graph (no re-binning since)";
            return 3;
        }
        if (phase == 2 && !kicked_) {
            err = "the drift phase follows a kick (phase 1) and a forces pass";
            return 3;
        }
        int rc;
        if (!wref_.rho) {
            const size_t n = (size_t)id_cap_;
            if ((rc = alloc(&wref_.rho, n, err)) || (rc = alloc(&wref_.v, n, err)) ||
                (rc = alloc(&wref_.drho, n, err)) || (rc = alloc(&wref_.a, n, err)) ||
                (rc = alloc(&wout_, 7, err)) || (rc = alloc(&ymean_, 3, err)))
                return rc;
        }
        const double *ym = nullptr;
        if (zero_momentum && phase != 2) {
            TSPH_CK(cudaMemsetAsync(ymean_, 0, 3 * sizeof(double), st_));
            if ((rc = launch(CAT_OTHER, k_fluid_sum2, blocks_for(nf_), kBlock, err,
                             (const uint32_t *)fstart_, ncells_, nw_, y, ymean_)))
                return rc;
            ym = ymean_;
        }
        if ((rc = launch(CAT_OTHER, k_apply_update<T>, blocks_for(nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, nw_, y, (float)su, (float)ss, kdt,
                         add_rates ? 1 : 0, phase, ym, P_.rho0, wref_, health_)))
            return rc;
        kicked_ = phase == 1;
        if (phase != 1) {
            cells_ = false;
            exported_ = false;
        }
        return collect_profile(err);
    }

    int window_check(double kdt, double out[5], std::string &err) override {
        TSPH_FRESH_P(err);
        if (!wref_.rho) {
            err = "no surrogate window was applied";
            return 3;
        }
        if (!cells_ok()) {
            err = "cell lists are stale: the check follows a forces pass at the window's end";
            return 3;
        }
        int rc;
        TSPH_CK(cudaMemsetAsync(wout_, 0, 7 * sizeof(double), st_));
        if ((rc = launch(CAT_OTHER, k_window_check<T>, blocks_for(nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, kdt, P_.rho0, wref_, wout_)))
            return rc;
        double h[7];
        TSPH_CK(cudaMemcpyAsync(h, wout_, sizeof h, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        const double rho0 = (double)P_.rho0, cnt = h[5] > 0 ? h[5] : 1.0;
        out[0] = h[0] / rho0;
        out[1] = std::sqrt(h[1] / cnt) / rho0;
        // momentum error per particle against gravity's impulse over the window
        const double gk = (double)P_.g * kdt * cnt;
        out[2] = std::sqrt(h[2] * h[2] + h[3] * h[3]) / (gk > 0 ? gk : 1e-300);
        out[3] = h[5];
        unsigned long long w;
        std::memcpy(&w, &h[6], 8);
        out[4] = (double)(uint32_t)(w & 0xffffffffull);
        return collect_profile(err);
    }

    // BZ_Integrate_inlet, src/SPH_buffer_zones.h:10-108
    int bz_inlet(int zone, double dt, std::string &err) override {
        TSPH_FRESH_P(err);
        if (!zones_on_ || zone < 0 || zone >= (int)zones_.size()) {
            err = "no such buffer zone";
            return 1;
        }
        const ZoneDev Z = zones_[zone];
        int rc;
        TSPH_CK(cudaMemsetAsync(zcount_, 0, 4, st_));
        if ((rc = launch(CAT_OTHER, k_inlet_cross<T>, blocks_for(nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, Z, dt, zlist_, zlist_cap_, zcount_)))
            return rc;
        uint32_t h[2] = {0, 0};
        TSPH_CK(cudaMemcpyAsync(&h[0], zcount_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaMemcpyAsync(&h[1], fstart_ + ncells_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        const int k = (int)h[0];
        if (k == 0) return collect_profile(err);
        if (k > zlist_cap_ || (int)h[1] + k > nf_ || ntot_ + k > id_cap_) {
            err = "buffer zone: no room for the particles the inlet creates (rows " +
                  std::to_string(h[1]) + " + " + std::to_string(k) + " of " + std::to_string(nf_) +
                  ", indices " + std::to_string(ntot_) + " of " + std::to_string(id_cap_) + ")";
            return 4;
        }
        if ((rc = launch(CAT_OTHER, k_inlet_append<T>, blocks_for(k), kBlock, err, F_, O_,
                         (const uint32_t *)fstart_, ncells_, Z, (const uint32_t *)zlist_, k,
                         (uint32_t)ntot_, P_.rho0, dt)) ||
            (rc = launch(CAT_OTHER, k_grow_live, 1, 32, err, fstart_, ncells_, k)))
            return rc;
        ntot_ += k;
        cells_ = false;
        return collect_profile(err);
    }

    // BZ_Integrate_outlet, src/SPH_buffer_zones.h:111-206 (x zones; the
    // reference's y branches are empty)
    int bz_outlet(int zone, double dt, std::string &err) override {
        TSPH_FRESH_P(err);
        (void)dt;
        if (!zones_on_ || zone < 0 || zone >= (int)zones_.size()) {
            err = "no such buffer zone";
            return 1;
        }
        const ZoneDev Z = zones_[zone];
        if (Z.ox == 0) return 0;
        int rc;
        TSPH_CK(cudaMemsetAsync(zlive_, 0, (size_t)ntot_, st_));
        TSPH_CK(cudaMemsetAsync(zcand_, 0, (size_t)ntot_, st_));
        TSPH_CK(cudaMemsetAsync(removed_, 0, 4, st_));
        if ((rc = launch(CAT_OTHER, k_outlet_mark<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, (const uint32_t *)W_.id, nw_, Z, zlive_,
                         zcand_)) ||
            (rc = launch(CAT_OTHER, k_outlet_apply<T>, blocks_for(nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, Z, (const uint8_t *)zlive_,
                         (const uint8_t *)zcand_, removed_, health_)))
            return rc;
        cells_ = false;
        return collect_profile(err);
    }

    int state_save(std::string &err) override {
        TSPH_FRESH_P(err);
        int rc;
        const size_t n = (size_t)nf_, nw = (size_t)nw_;
        if (!saved_) {
            if ((rc = alloc(&Fsv_.r, n, err)) || (rc = alloc(&Fsv_.v, n, err)) ||
                (rc = alloc(&Fsv_.a, n, err)) || (rc = alloc(&Fsv_.rho, n, err)) ||
                (rc = alloc(&Fsv_.drho, n, err)) || (rc = alloc(&Fsv_.p, n, err)) ||
                (rc = alloc(&Fsv_.id, n, err)) || (rc = alloc(&Fsv_.key, n, err)) ||
                (rc = alloc(&Fsv_.loc, n, err)) || (rc = alloc(&wsv_, 4 * nw, err)) ||
                (F_.type && (rc = alloc(&Fsv_.type, n, err))) ||
                (rc = alloc(&fstart_sv_, (size_t)ncells_ + 1, err)) ||
                (rc = alloc(&lbin_sv_, n, err)) || (rc = alloc(&gen_sv_, 4, err)))
                return rc;
        }
        // the kept-list state goes with it (restored when no kept-list pass
        // ran in between, so stepping on from the restored state is the same
        // as stepping on from the saved one)
        TSPH_CK(cudaMemcpyAsync(lbin_sv_, lbin_, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st_));
        TSPH_CK(cudaMemcpyAsync(gen_sv_, gen_, 16, cudaMemcpyDeviceToDevice, st_));
        rec_passes_sv_ = rec_passes_;
        copy_state(Fsv_, F_, wsv_, false);
        TSPH_CK(cudaMemcpyAsync(fstart_sv_, fstart_, 4 * ((size_t)ncells_ + 1),
                                cudaMemcpyDeviceToDevice, st_));
        TSPH_CK(cudaGetLastError());
        saved_ = true;
        saved_cells_ = cells_;
        saved_kept_ = cells_kept_;
        return 0;
    }

    int state_restore(std::string &err) override {
        if (!saved_) {
            err = "no saved state";
            return 3;
        }
        p_stale_ = false;  // the saved pressure was brought up to date by state_save
        copy_state(F_, Fsv_, wsv_, true);
        TSPH_CK(cudaMemcpyAsync(fstart_, fstart_sv_, 4 * ((size_t)ncells_ + 1),
                                cudaMemcpyDeviceToDevice, st_));
        TSPH_CK(cudaGetLastError());
        cells_ = saved_cells_;
        cells_kept_ = saved_kept_;
        exported_ = false;
        kicked_ = false;
        TSPH_CK(cudaMemcpyAsync(lbin_, lbin_sv_, sizeof(float2) * (size_t)nf_,
                                cudaMemcpyDeviceToDevice, st_));
        TSPH_CK(cudaMemcpyAsync(gen_, gen_sv_, 16, cudaMemcpyDeviceToDevice, st_));
        // the window table of the restored cells (a binning since the save
        // may have rebuilt it for other cells)
        int rc;
        if ((rc = pair_records(F_, nullptr, true, err))) return rc;
        if (rec_passes_ == rec_passes_sv_) return 0;  // the lists are the saved state's
        // lists rebuilt since the save: when the saved state's were current,
        // build them again at its binning positions (the same lists), else
        // leave them stale as they were
        if constexpr (std::is_same<T, float>::value) {
            uint32_t g[4];
            TSPH_CK(cudaMemcpyAsync(g, gen_sv_, 16, cudaMemcpyDeviceToHost, st_));
            TSPH_CK(cudaStreamSynchronize(st_));
            if (g[0] == g[1] && rec_f_.e && tile_shape_ == 2) {
                if ((rc = launch(CAT_OTHER, k_lbin_records, blocks_for(nf_), kBlock, err, rec_f_,
                                 (const float2 *)lbin_, (const uint32_t *)F_.key,
                                 (const uint32_t *)fstart_, grid_)))
                    return rc;
                return fluid_pairs_rec<MODE_LISTS>(F_, T(0), PairOut{}, err, 0, false);
            }
        }
        return mark_stale(err);
    }

    int set_tile_shape(int shape, std::string &err) override {
        TSPH_FRESH_P(err);
        if (shape < 0 || shape >= kShapes) {
            err = "tile shape must be 0, 1 or 2";
            return 1;
        }
        if (cases_on_ && shape != 2) {
            err = "packed cases: the pair-record kernel (shape 2) only";
            return 1;
        }
        tile_shape_ = shape;
        for (auto &g : graphs_) cudaGraphExecDestroy(g.second);
        graphs_.clear();
        return 0;
    }

  private:
    // fluid rows and the evolving wall fields, between the live state and the
    // saved copy (to_live: saved -> live)
    void copy_state(FluidState<T> &dst, const FluidState<T> &src, T *wsv, bool to_live) {
        const size_t n = (size_t)nf_, nw = (size_t)nw_;
        const auto D = cudaMemcpyDeviceToDevice;
        cudaMemcpyAsync(dst.r, src.r, 16 * n, D, st_);
        cudaMemcpyAsync(dst.v, src.v, sizeof(T2) * n, D, st_);
        cudaMemcpyAsync(dst.a, src.a, sizeof(T2) * n, D, st_);
        cudaMemcpyAsync(dst.rho, src.rho, sizeof(T) * n, D, st_);
        cudaMemcpyAsync(dst.drho, src.drho, sizeof(T) * n, D, st_);
        cudaMemcpyAsync(dst.p, src.p, sizeof(T) * n, D, st_);
        cudaMemcpyAsync(dst.id, src.id, 4 * n, D, st_);
        cudaMemcpyAsync(dst.key, src.key, 4 * n, D, st_);
        cudaMemcpyAsync(dst.loc, src.loc, 8 * n, D, st_);
        if (dst.type && src.type) cudaMemcpyAsync(dst.type, src.type, n, D, st_);
        T *wl[4] = {W_.rho, W_.drho, W_.p, W_.rho_o};
        for (int k = 0; k < 4; k++) {
            if (to_live) cudaMemcpyAsync(wl[k], wsv + k * nw, sizeof(T) * nw, D, st_);
            else cudaMemcpyAsync(wsv + k * nw, wl[k], sizeof(T) * nw, D, st_);
        }
    }


    // the fluid-row pair pass: tiled FP32 kernel, or the plain FP64 kernel.
    // `skinned`: the cells are those of the binning before the predictor.
    template <int MODE>
    int fluid_pairs(const FluidState<T> &X, bool stored_p, T dt, PairOut po, std::string &err,
                    bool skinned = false) {
        if (wall_model_ == 2)  // boundary-integral walls: the per-particle kernel
            return launch(CAT_PAIR, k_fluid_pairs<T, MODE, true>, blocks_for(nf_), kBlock, err, X,
                          (const uint32_t *)fstart_, (const uint32_t *)wstart_,
                          nbr_fluid(X, stored_p), nbr_walls_bt(stored_p), grid_, P_, O_, dt, po,
                          health_, (int32_t *)nullptr, (long long *)nullptr, (int32_t *)nullptr,
                          (const uint32_t *)nullptr);
        if (zones_on_)  // buffer particles: the per-particle kernel skips them as targets
            return launch(CAT_PAIR, k_fluid_pairs<T, MODE, false>, blocks_for(nf_), kBlock, err, X,
                          (const uint32_t *)fstart_, (const uint32_t *)wstart_,
                          nbr_fluid(X, stored_p), nbr_walls(stored_p), grid_, P_, O_, dt, po,
                          health_, (int32_t *)nullptr, (long long *)nullptr, (int32_t *)nullptr,
                          (const uint32_t *)nullptr);
        if constexpr (std::is_same<T, float>::value) {
            const int nb = blocks_for(nf_, kTileT);
            const TileConst K = skinned ? Kskin_ : K_;
            const uint32_t *fs = fstart_, *ws = wstart_;
            // shape 2 keeps its lists only inside the fused step (fluid_pairs_rec);
            // every other pair pass takes the faster tiled shape
            const int shape = tile_shape_ == 2 ? tiled_best_ : tile_shape_;
            if (shape == 1) {
                if (stored_p)
                    return launch(CAT_PAIR, k_pairs_tiled<MODE, true, TileDeep>, nb, kTileT, err,
                                  X, fs, ws, W_, grid_, P_, K, O_, dt, po, health_);
                return launch(CAT_PAIR, k_pairs_tiled<MODE, false, TileDeep>, nb, kTileT, err, X,
                              fs, ws, W_, grid_, P_, K, O_, dt, po, health_);
            }
            if (stored_p)
                return launch(CAT_PAIR, k_pairs_tiled<MODE, true, TileWide>, nb, kTileT, err, X,
                              fs, ws, W_, grid_, P_, K, O_, dt, po, health_);
            return launch(CAT_PAIR, k_pairs_tiled<MODE, false, TileWide>, nb, kTileT, err, X, fs,
                          ws, W_, grid_, P_, K, O_, dt, po, health_);
        } else {
            return launch(CAT_PAIR, k_fluid_pairs<T, MODE>, blocks_for(nf_), kBlock, err, X,
                          (const uint32_t *)fstart_, (const uint32_t *)wstart_,
                          nbr_fluid(X, stored_p), nbr_walls(stored_p), grid_, P_, O_, dt, po,
                          health_, (int32_t *)nullptr, (long long *)nullptr, (int32_t *)nullptr,
                          (const uint32_t *)nullptr);
        }
    }

    // the pair pass over pair records with kept lists (shape 2, the fused
    // step and the autotuner): the records kernel forms X's records and the
    // window table and decides whether this pass builds the lists (a sort
    // happened since they were built) or sums the stored ones
    template <int MODE>
    int fluid_pairs_rec(const FluidState<T> &X, T dt, PairOut po, std::string &err,
                        cudaGraphConditionalHandle cond_sort = 0, bool records = true) {
        if constexpr (std::is_same<T, float>::value) {
            int rc;
            if (!rec_setup_) {
                const void *kr[5] = {(const void *)k_pairs_rec<MODE_FORCES, false, RecStd>,
                                     (const void *)k_pairs_rec<MODE_CORRECT, false, RecStd>,
                                     (const void *)k_pairs_rec<MODE_LISTS, false, RecStd>,
                                     (const void *)k_pairs_rec<MODE_FORCES, false, RecStd, true>,
                                     (const void *)k_pairs_rec<MODE_CORRECT, false, RecStd, true>};
                for (const void *k : kr)
                    TSPH_CK(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                 (int)cudaSharedmemCarveoutMaxShared));
                rec_setup_ = true;
            }
            rec_passes_++;
            const uint32_t *fs = fstart_, *ws = wstart_;
            const PairRec RX = X.r == Fs_.r ? rec_s_ : rec_f_;
            const int nchunks = blocks_for(nf_, kRecT);
            if (records && (rc = pair_records(X, nullptr, false, err))) return rc;
            // MODE_CORRECT writes the new state into F_ in the kept order,
            // with its cell-relative positions and the next pass's records
            RecStep S{rec_list_, rec_cnt_, gen_, (const float2 *)lbin_, sig2_, F_.loc, rec_f_,
                      need_sort_, cond_sort, capturing_ ? 1 : 0, col_case_, cases_};
            // the corrector's old state: F_ itself (the predictor leaves it
            // in place; the pass overwrites each row after reading it)
            const OldState<T> OF{F_.r, F_.v, F_.rho};
            if constexpr (MODE != MODE_LISTS)  // (list building reads no case constant)
                if (cases_on_)
                    return launch(CAT_PAIR, k_pairs_rec<MODE, false, RecStd, true>, nchunks,
                                  kRecT, err, X, fs, ws, W_, grid_, P_, Krec_, Krec_build_, OF, dt,
                                  po, RX, rec_w_, (const WinRec *)rec_table_,
                                  (const int *)rec_nwin_, S, health_);
            return launch(CAT_PAIR, k_pairs_rec<MODE, false, RecStd>, nchunks, kRecT, err, X, fs, ws,
                          W_, grid_, P_, Krec_, Krec_build_, OF, dt, po, RX, rec_w_,
                          (const WinRec *)rec_table_, (const int *)rec_nwin_, S, health_);
        } else {
            (void)X;
            (void)dt;
            (void)po;
            (void)cond_sort;
            (void)records;
            err = "pair records: FP32 build only";
            return 8;
        }
    }

    // the neighbour lists of F_ at its binned positions (MODE_LISTS pass,
    // records of F_ already formed), for systems whose fused step keeps them
    int build_lists(std::string &err) {
        if constexpr (std::is_same<T, float>::value) {
            if (!rec_f_.e || tile_shape_ != 2 || skin_ <= 0.f || wall_model_ == 2 || zones_on_)
                return 0;
            int rc;
            return fluid_pairs_rec<MODE_LISTS>(F_, T(0), PairOut{}, err, 0, false);
        } else {
            (void)err;
            return 0;
        }
    }

    // the pair records of state X (fluid rows and walls) and, after a sort
    // (or when forced), the window table: for passes whose records no
    // producer wrote (after a binning, the autotuner)
    int pair_records(const FluidState<T> &X, const uint32_t *gate, bool force_table,
                     std::string &err) {
        if constexpr (std::is_same<T, float>::value) {
            if (!rec_f_.e) return 0;
            const PairRec RX = X.r == Fs_.r ? rec_s_ : rec_f_;
            const int nchunks = blocks_for(nf_, kRecT);
            const int rb = blocks_for((long long)nw_ + nf_);
            const int tb = rb + blocks_for(nchunks);
            // the records kernel is timed apart from the pair kernel (CAT_OTHER)
            return launch(CAT_OTHER, k_pair_records<false>, tb, kBlock, err, X,
                          (const uint32_t *)fstart_, W_, nw_, grid_, P_, RX, rec_w_, rb,
                          (const uint32_t *)wstart_, nchunks, RecStd::cap, rec_table_, rec_nwin_,
                          gen_, gate, force_table ? 1 : 0);
        } else {
            (void)X;
            (void)gate;
            (void)force_table;
            (void)err;
            return 0;
        }
    }

    // cells kept over several steps are re-binned at the current positions
    // before anything that needs the reference's cells (tiled pair passes,
    // cell lists, pair digests)
    int ensure_exact_cells(std::string &err) {
        if (!cells_kept_) return 0;
        return bin_particles(err, false);
    }

  public:
    int settle_cells(std::string &err) override {
        TSPH_FRESH_P(err);
        return ensure_exact_cells(err);
    }

  private:
    // the state changed outside the fused step: neighbour lists and binning
    // positions are stale (the next fused step re-bins first)
    int mark_stale(std::string &err) {
        TSPH_CK(cudaMemsetAsync(gen_ + 1, 0xff, 4, st_));
        return 0;
    }

    // re-binning of the predicted state Fs_ (+ old state O_): sort into F_
    // and B, copy back (FP32 fused step, when the skin was exceeded)
    // With `rec` (the fused step over pair records) the old state lives in
    // F_ itself (the predictor writes no O_): it is copied into O_ to be
    // carried through the sort and lands back in F_.
    int rebin_predicted(const uint32_t *gate, T dt, bool rec, std::string &err) {
        int rc;
        const OldState<T> FO{F_.r, F_.v, F_.rho};
        if ((rc = launch(CAT_SORT, k_predict_r<T>, blocks_for(nf_), kBlock, err, Fs_,
                         rec ? FO : O_, O_, (const uint32_t *)fstart_, ncells_, dt, gate,
                         rec ? 1 : 0)))
            return rc;
        if ((rc = launch(CAT_SORT, k_bin_gated<T>, blocks_for(nf_), kBlock, err,
                         (const FluidState<T>)Fs_, (const uint32_t *)fstart_, grid_, keyB_, slotB_,
                         counts_, health_, gate, body_ == 1 ? body_runs_ + 1 : (uint32_t *)nullptr)))
            return rc;
        if ((rc = sort_finish(Fs_.r, Fs_.v, Fs_.rho, Fs_.id, nullptr, nullptr, nullptr, F_, O_.r,
                              O_.v, O_.rho, OldState<T>{Br_, Bv_, Brho_}, err, gate)))
            return rc;
        return launch(CAT_SORT, k_copy_back<T>, blocks_for(nf_), kBlock, err,
                      (const FluidState<T>)F_, (const double2 *)Br_, (const T2 *)Bv_,
                      (const T *)Brho_, (const uint32_t *)fstart_, ncells_, Fs_, rec ? FO : O_,
                      gate);
    }

    // during capture: an IF node on `cond` after the current work, its body
    // captured from `body` (kernels counted as conditional body `id`)
    template <typename F>
    int add_cond_body(cudaGraphConditionalHandle cond, int id, const char *what, F body,
                      std::string &err) {
        cudaGraph_t cg = nullptr;
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t *deps = nullptr;
        size_t nd = 0;
        TSPH_CK(cudaStreamGetCaptureInfo(st_, &cs, nullptr, &cg, &deps, nullptr, &nd));
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = cond;
        np.conditional.type = cudaGraphCondTypeIf;
        np.conditional.size = 1;
        cudaGraphNode_t cn;
        TSPH_CK(cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &np));
        cudaGraph_t g = np.conditional.phGraph_out[0];
        if (!st2_) TSPH_CK(cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking));
        TSPH_CK(cudaStreamBeginCaptureToGraph(st2_, g, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal));
        std::swap(st_, st2_);
        body_ = id;
        int rc = body();
        body_ = 0;
        std::swap(st_, st2_);
        cudaGraph_t bodyc = nullptr;
        const cudaError_t e = cudaStreamEndCapture(st2_, &bodyc);
        if (rc) return rc;
        if (e != cudaSuccess) {
            err = std::string("cudaStreamEndCapture (") + what + "): " + cudaGetErrorString(e);
            return 2;
        }
        TSPH_CK(cudaStreamUpdateCaptureDependencies(st_, &cn, nullptr, 1,
                                                    cudaStreamSetCaptureDependencies));
        return 0;
    }

    // one fused step (enqueue only)
    int enqueue_step(int model, T dt, std::string &err) {
        int rc;
        const bool dbc = model == 1;
        wall_model_ = model;
        bool skinned = false;
        if constexpr (std::is_same<T, float>::value) skinned = skin_ > 0.f;
        // FP32 mDBC step with the skin: mDBC and the predictor share a launch
        const bool mdbc_fused = model == 0 && nw_ > 0 && skinned;
        // pair records with kept lists (shape 2): the cells are kept over
        // several steps, re-binned after the predictor when a particle moved
        // sigma since its binning or the lists are stale, and after the
        // corrector when a particle moved sigma or left the domain
        const bool rec = skinned && tile_shape_ == 2 && model != 2 && !zones_on_;
        const KeepCells kc = rec ? KeepCells{(const float2 *)lbin_, sig2_, gen_, need_sort_}
                                 : KeepCells{nullptr, 0.f, nullptr, nullptr};
        if (model == 0 && !mdbc_fused && (rc = do_mdbc(err))) return rc;
        if (model == 2 && (rc = do_bt_density(err))) return rc;
        if (skinned) {
            // predictor in the current order; the re-binning runs only when
            // some particle moved more than the skin: in a graph as the body
            // of a conditional node the predictor switches on, otherwise as
            // kernels gated on rebuild_ (which only that gating reads: a
            // graph step needs no memset node for it)
            if (!capturing_) TSPH_CK(cudaMemsetAsync(rebuild_, 0, 4, st_));
            cudaGraphConditionalHandle cond = 0;
            cudaGraph_t cg = nullptr;
            cudaStreamCaptureStatus cs;
            const cudaGraphNode_t *deps = nullptr;
            size_t nd = 0;
            if (capturing_) {
                TSPH_CK(cudaStreamGetCaptureInfo(st_, &cs, nullptr, &cg, &deps, nullptr, &nd));
                TSPH_CK(cudaGraphConditionalHandleCreate(&cond, cg, 0, cudaGraphCondAssignDefault));
            }
            if constexpr (std::is_same<T, float>::value) {
                if (mdbc_fused) {
                    const int lanes = mdbc_lanes(nw_, sm_count_);
                    const int nbm = blocks_for((long long)nw_ * lanes);
                    // walls needing more than one wave (4 blocks per SM)
                    // share their waves with the predictor's blocks
                    const int inter = nbm > 4 * sm_count_ ? 1 : 0;
                    rc = launch(CAT_MDBC, lanes == kMdbcLanes ? k_mdbc_f32_predict<kMdbcLanes>
                                                              : k_mdbc_f32_predict<kMdbcLanesMany>,
                                nbm + blocks_for((nf_ + kPredU - 1) / kPredU), kBlock, err, W_,
                                nw_, nbm, (const uint32_t *)fstart_, F_, grid_, P_, dt, Fs_, O_,
                                skin_, rebuild_, health_, cond, capturing_ ? 1 : 0, kc,
                                rec ? rec_s_ : PairRec{}, rec ? rec_w_ : PairRec{}, inter);
                    if (rc) return rc;
                }
            }
            if (!mdbc_fused &&
                (rc = launch(CAT_OTHER, k_predict_keep<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                             (const uint32_t *)fstart_, W_, nw_, grid_, dt, Fs_, O_, skin_,
                             rebuild_, health_, cond, capturing_ ? 1 : 0, kc,
                             rec ? rec_s_ : PairRec{}, rec ? rec_w_ : PairRec{}, P_)))
                return rc;
            if (capturing_) {
                TSPH_CK(cudaStreamGetCaptureInfo(st_, &cs, nullptr, &cg, &deps, nullptr, &nd));
                cudaGraphNodeParams np = {};
                np.type = cudaGraphNodeTypeConditional;
                np.conditional.handle = cond;
                np.conditional.type = cudaGraphCondTypeIf;
                np.conditional.size = 1;
                cudaGraphNode_t cn;
                TSPH_CK(cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &np));
                cudaGraph_t body = np.conditional.phGraph_out[0];
                if (!st2_) TSPH_CK(cudaStreamCreateWithFlags(&st2_, cudaStreamNonBlocking));
                TSPH_CK(cudaStreamBeginCaptureToGraph(st2_, body, nullptr, nullptr, 0,
                                                      cudaStreamCaptureModeThreadLocal));
                std::swap(st_, st2_);
                body_ = 1;
                rc = rebin_predicted(nullptr, dt, rec, err);
                if (!rc && rec) rc = pair_records(Fs_, nullptr, false, err);
                body_ = 0;
                std::swap(st_, st2_);
                cudaGraph_t bodyc = nullptr;
                const cudaError_t e = cudaStreamEndCapture(st2_, &bodyc);
                if (rc) return rc;
                if (e != cudaSuccess) {
                    err = std::string("cudaStreamEndCapture (re-binning body): ") +
                          cudaGetErrorString(e);
                    return 2;
                }
                TSPH_CK(cudaStreamUpdateCaptureDependencies(st_, &cn, nullptr, 1,
                                                            cudaStreamSetCaptureDependencies));
            } else if ((rc = rebin_predicted(rebuild_, dt, rec, err)) ||
                       (rec && (rc = pair_records(Fs_, rebuild_, false, err)))) {
                return rc;
            }
        } else {
            // predictor + bin
            if ((rc = zero_counts(err))) return rc;
            if ((rc = launch(CAT_OTHER, k_predict_bin<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                             (const uint32_t *)fstart_, W_, nw_, grid_, dt, Br_, Bv_, Brho_, keyB_,
                             slotB_, counts_, health_)))
                return rc;
            if ((rc = sort_finish(Br_, Bv_, Brho_, F_.id, nullptr, nullptr, nullptr, Fs_, F_.r,
                                  F_.v, F_.rho, O_, err)))
                return rc;
        }
        // forces at the predicted state + corrector + bin
        if ((rc = zero_counts(err))) return rc;
        PairOut po{Br_, (void *)Bv_, (void *)Brho_, keyB_, slotB_, counts_, box_, make_box_bits(box_)};
        po.rm = Removal{rm_cand_, rm_list_, rm_count_, kRemovalCap, (const uint32_t *)Fs_.id};
        // the erase of the corrector's candidates, before the sort
        auto resolve = [&](const uint32_t *gate) -> int {
            return launch(CAT_SORT, k_resolve_removal, 1, kResolveThreads, err, po.rm, dead_, keyB_,
                          slotB_, counts_, ncells_, health_, gate);
        };
        auto wall_rows = [&](PairRec RW) -> int {
            if (nw_ == 0) return 0;
            return launch(CAT_OTHER, k_wall_rows<T>, blocks_for(nw_), kBlock, err, W_, nw_,
                          (const uint32_t *)fstart_, nbr_fluid(Fs_, false), grid_, P_, dbc, true, dt,
                          (int32_t *)nullptr, (long long *)nullptr, (int32_t *)nullptr,
                          (const uint32_t *)nullptr, false, RW);
        };
        auto sort_new = [&](const uint32_t *gate, uint32_t *runs) -> int {
            return sort_finish(Br_, Bv_, Brho_, Fs_.id, nullptr, nullptr, nullptr, F_, nullptr,
                               nullptr, nullptr, O_, err, gate, nullptr, runs);
        };
        if (rec) {
            // The corrector writes the new state into F_ in the kept order,
            // with the next pass's pair records (the walls' from k_wall_rows).
            // Only when some particle left its kept cell's reach or the
            // domain does the sort run: histogram, erase, sort of F_ into Fs_,
            // rows copied back, records and window table of the new order
            // (a conditional node in a graph, kernels gated on need_sort_
            // otherwise).
            cudaGraphConditionalHandle cs_ = 0;
            if (capturing_) {
                cudaGraph_t cg = nullptr;
                cudaStreamCaptureStatus cst;
                TSPH_CK(cudaStreamGetCaptureInfo(st_, &cst, nullptr, &cg, nullptr, nullptr, nullptr));
                TSPH_CK(cudaGraphConditionalHandleCreate(&cs_, cg, 0, cudaGraphCondAssignDefault));
            }
            PairOut pk{F_.r, (void *)F_.v, (void *)F_.rho, keyB_, slotB_, counts_, box_,
                       make_box_bits(box_)};
            pk.rm = Removal{rm_cand_, rm_list_, rm_count_, kRemovalCap, (const uint32_t *)F_.id};
            if ((rc = fluid_pairs_rec<MODE_CORRECT>(Fs_, dt, pk, err, cs_, false))) return rc;
            if ((rc = wall_rows(rec_w_))) return rc;
            auto sort_kept = [&](const uint32_t *gate, uint32_t *runs) -> int {
                int r;
                if ((r = launch(CAT_SORT, k_hist_kept<T>, blocks_for(nf_), kBlock, err,
                                (const FluidState<T>)F_, keyB_, slotB_, counts_,
                                (const uint8_t *)rm_cand_, (const uint32_t *)fstart_, grid_,
                                make_box_bits(box_), health_, gate, runs,
                                (const int32_t *)col_case_, (const CaseConst *)cases_)) ||
                    (r = launch(CAT_SORT, k_resolve_removal, 1, kResolveThreads, err, pk.rm, dead_,
                                keyB_, slotB_, counts_, ncells_, health_, gate)) ||
                    (r = sort_finish(F_.r, F_.v, F_.rho, F_.id, nullptr, nullptr, nullptr, Fs_,
                                     nullptr, nullptr, nullptr, O_, err, gate)) ||
                    (r = launch(CAT_SORT, k_copy_rows<T>, blocks_for(nf_), kBlock, err, F_,
                                (const FluidState<T>)Fs_, (const uint32_t *)fstart_, ncells_,
                                gate)) ||
                    (r = pair_records(F_, gate, false, err)))
                    return r;
                return 0;
            };
            if (capturing_) {
                if ((rc = add_cond_body(cs_, 2, "sort body",
                                        [&]() { return sort_kept(nullptr, body_runs_ + 2); },
                                        err)))
                    return rc;
            } else if ((rc = sort_kept(need_sort_, nullptr))) {
                return rc;
            }
            // forces at the new state (a, drho for the next predictor)
            if ((rc = fluid_pairs_rec<MODE_FORCES>(F_, dt, PairOut{}, err, 0, false))) return rc;
            if (dbc && nw_ > 0 &&
                (rc = launch(CAT_OTHER, k_wall_rows<T>, blocks_for(nw_), kBlock, err, W_, nw_,
                             (const uint32_t *)fstart_, nbr_fluid(F_, false), grid_, P_, true, false,
                             dt, (int32_t *)nullptr, (long long *)nullptr, (int32_t *)nullptr,
                             (const uint32_t *)nullptr, false, PairRec{})))
                return rc;
            return 0;
        }
        if ((rc = fluid_pairs<MODE_CORRECT>(Fs_, false, dt, po, err, skinned))) return rc;
        if ((rc = wall_rows(PairRec{}))) return rc;
        if ((rc = resolve(nullptr))) return rc;
        if ((rc = sort_new(nullptr, nullptr))) return rc;
        // forces at the new state (a, drho for the next predictor)
        if ((rc = fluid_pairs<MODE_FORCES>(F_, false, dt, PairOut{}, err))) return rc;
        if (dbc && nw_ > 0 &&
            (rc = launch(CAT_OTHER, k_wall_rows<T>, blocks_for(nw_), kBlock, err, W_, nw_,
                         (const uint32_t *)fstart_, nbr_fluid(F_, false), grid_, P_, true, false, dt,
                         (int32_t *)nullptr, (long long *)nullptr, (int32_t *)nullptr,
                         (const uint32_t *)nullptr, false, PairRec{})))
            return rc;
        return 0;
    }

  public:
    ~Engine() override {
        if (cs_) cudaStreamSynchronize(cs_);  // a download still in flight
        if (cs_) cudaStreamDestroy(cs_);
        if (ev_x_) cudaEventDestroy(ev_x_);
        if (ev_d_) cudaEventDestroy(ev_d_);
        if (cu_) cudaStreamSynchronize(cu_);  // a staged upload's copies
        if (cu_) cudaStreamDestroy(cu_);
        if (ev_up_) cudaEventDestroy(ev_up_);
        if (ev_imp_) cudaEventDestroy(ev_imp_);
        for (auto &g : graphs_) cudaGraphExecDestroy(g.second);
        for (auto &m : marks_) {
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
        for (auto e : ev_pool_) cudaEventDestroy(e);
        for (void *p : allocs_) cudaFree(p);
        if (pr_d_) cudaFree(pr_d_);
        if (st2_) cudaStreamDestroy(st2_);
        if (own_stream_ && st_) cudaStreamDestroy(st_);
    }

    int init(const HostSetup &hs, void *stream, std::string &err) override {
        if (const char *v = std::getenv("TSPH_PDL")) pdl_ = std::atoi(v) != 0;
        {
            int dev = 0, sms = 0;
            TSPH_CK(cudaGetDevice(&dev));
            TSPH_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            if (sms > 0) sm_count_ = sms;
        }
        if (stream) {
            st_ = static_cast<cudaStream_t>(stream);
        } else {
            TSPH_CK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
            own_stream_ = true;
        }
        const int n = (int)hs.type.size();
        ntot_ = n;
        ncells_ = hs.ncx * hs.ncy;
        // split fluid / walls
        std::vector<int> fl, wl;
        for (int i = 0; i < n; i++) (hs.type[i] == 1 ? wl : fl).push_back(i);
        zones_on_ = !hs.zones.empty();
        const int nf0 = (int)fl.size();
        nf_ = nf0 + (zones_on_ ? hs.extra_rows : 0);
        nw_ = (int)wl.size();
        id_cap_ = ntot_ + (zones_on_ ? hs.extra_ids : 0);
        for (size_t z = 0; z + 12 <= hs.zones.size(); z += 12) {
            const double *q = hs.zones.data() + z;
            ZoneDev d;
            d.ox = q[0];
            d.oy = q[1];
            d.x_b = q[0] != 0 ? q[2] : q[3];
            d.b_len = q[7];
            d.btype = (int)q[9];
            d.vbx = q[10];
            d.vby = q[11];
            d.dp = hs.dp;
            zones_.push_back(d);
        }
        // constants
        m64_ = hs.m;
        dp64_ = hs.dp;
        P_.hd = hs.h;
        P_.h = (T)hs.h;
        P_.inv_h = (T)(1.0 / hs.h);
        P_.kh = (T)hs.kh;
        P_.m = (T)hs.m;
        P_.c0 = (T)hs.cs;
        P_.alpha = (T)hs.visco;
        P_.delta = (T)hs.delta;
        P_.rho0 = (T)hs.rho0;
        P_.g = (T)hs.g;
        P_.dp = (T)hs.dp;
        P_.awen = (T)(double)(float)(0.557 / (hs.h * hs.h));
        P_.bwen = (T)(double)(float)(-2.7852 / (hs.h * hs.h * hs.h));
        P_.four_h2 = (T)(4.0 * hs.h * hs.h);
        P_.eps_h2 = (T)(0.01 * hs.h * hs.h);
        P_.bwen_h = (T)((double)(float)(-2.7852 / (hs.h * hs.h * hs.h)) / hs.h);
        P_.b_eos = (T)(hs.cs * hs.cs * hs.rho0 / 7.0);
        P_.k_av = (T)(-2.0 * hs.visco * hs.cs * hs.h);
        P_.k_psi = (T)(2.0 * hs.cs * hs.h * hs.delta);
        P_.xg = (T)(hs.rho0 * hs.g / (hs.cs * hs.cs * hs.rho0 / 7.0));
        box_ = Box{hs.x0, hs.xm, hs.y0, hs.ym};
        if constexpr (std::is_same<T, float>::value) {
            K_ = make_tile_const(P_, hs.h, hs.rho0, hs.g, hs.cs);
            // per-axis move allowed between two binnings: kh >= 2h + 2 skin,
            // with 5 % margin for the FP32 cell-local arithmetic
            skin_ = (float)(0.95 * 0.5 * (hs.kh - 2.0 * hs.h));
            Kskin_ = K_;
            Kskin_.reach = K_.reach + 2.f * skin_;
            // pair records: the support test and the window search use y in
            // the grid's frame (rounding up to half an ulp of the grid height
            // per value, plus the fma that forms it): 8 ulps of margin
            const double ytop = (double)hs.ncy * hs.kh;
            const float margin = 8.f * std::ldexp(1.f, std::ilogb((float)ytop) - 23);
            Krec_ = K_;
            Krec_.reach = K_.reach + margin;
            // kept cells: a re-binning is due once a particle has moved sigma
            // (Euclidean) from where it was binned; lists then hold the
            // neighbours within 2h + 2 sigma (<= kh: inside the 3 x 3 block)
            sig2_ = skin_ * skin_;
            const double rl = 2.0 * hs.h + 2.0 * (double)skin_;
            Krec_build_ = K_;
            Krec_build_.four_h2 = (float)(rl * rl);
            Krec_build_.reach = (float)(rl * 1.0001) + margin;
        }
        // grid tables
        int rc;
        if ((rc = alloc(&bx_, hs.bx.size(), err)) || (rc = alloc(&by_, hs.by.size(), err)) ||
            (rc = alloc(&ox_, hs.ox.size(), err)) || (rc = alloc(&oy_, hs.oy.size(), err)))
            return rc;
        TSPH_CK(cudaMemcpy(bx_, hs.bx.data(), 8 * hs.bx.size(), cudaMemcpyHostToDevice));
        TSPH_CK(cudaMemcpy(by_, hs.by.data(), 8 * hs.by.size(), cudaMemcpyHostToDevice));
        TSPH_CK(cudaMemcpy(ox_, hs.ox.data(), 8 * hs.ox.size(), cudaMemcpyHostToDevice));
        TSPH_CK(cudaMemcpy(oy_, hs.oy.data(), 8 * hs.oy.size(), cudaMemcpyHostToDevice));
        grid_.ax = Axis{bx_, ox_, hs.ncx};
        grid_.ay = Axis{by_, oy_, hs.ncy};
        grid_.ncx = hs.ncx;
        grid_.ncy = hs.ncy;
        grid_.ncells = ncells_;
        grid_.khf = (float)hs.kh;
        // fluid buffers
        auto alloc_state = [&](FluidState<T> &X) -> int {
            int r;
            if ((r = alloc(&X.r, nf_, err)) || (r = alloc(&X.v, nf_, err)) ||
                (r = alloc(&X.a, nf_, err)) || (r = alloc(&X.rho, nf_, err)) ||
                (r = alloc(&X.drho, nf_, err)) || (r = alloc(&X.p, nf_, err)) ||
                (r = alloc(&X.id, nf_, err)) || (r = alloc(&X.key, nf_, err)) ||
                (r = alloc(&X.loc, nf_, err)))
                return r;
            return 0;
        };
        if ((rc = alloc_state(F_)) || (rc = alloc_state(Fs_))) return rc;
        if constexpr (std::is_same<T, float>::value) {
            // pair records (tile shape 2): two 16-byte arrays per state, so
            // every window copy starts on a 16-byte boundary
            auto alloc_rec = [&](PairRec &R, int n) -> int {
                int r;
                const int cap = n + kRecPad;
                if ((r = alloc(&R.e, cap, err)) || (r = alloc(&R.v, cap, err)))
                    return r;
                return 0;
            };
            const int nchunks = blocks_for(nf_, kRecT);
            if ((rc = alloc_rec(rec_f_, nf_)) || (rc = alloc_rec(rec_s_, nf_)) ||
                (rc = alloc_rec(rec_w_, nw_)) ||
                (rc = alloc(&rec_table_, (size_t)nchunks * kRecMaxWin, err)) ||
                (rc = alloc(&rec_nwin_, nchunks, err)) ||
                (rc = alloc(&rec_list_, (size_t)nchunks * RecStd::list * kRecT, err)) ||
                (rc = alloc(&rec_cnt_, (size_t)nchunks * kRecT, err)))
                return rc;
        }
        if ((rc = alloc(&lbin_, nf_, err)) || (rc = alloc(&gen_, 4, err)) ||
            (rc = alloc(&need_sort_, 1, err)) || (rc = alloc(&pc_gate_, 1, err)))
            return rc;
        if (!hs.case_g.empty()) {
            if constexpr (std::is_same<T, float>::value) {
                if (!hs.zones.empty()) {
                    err = "packed cases: no buffer zones";
                    return 1;
                }
                if ((rc = setup_cases(hs, err))) return rc;
            } else {
                err = "packed cases: FP32 build only";
                return 8;
            }
        }
        {
            const uint32_t g0[4] = {1u, 0u, 0u, 0u};  // no lists yet: stale
            TSPH_CK(cudaMemcpy(gen_, g0, 16, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemset(need_sort_, 0, 4));
        }
        if (zones_on_) {
            zlist_cap_ = 1 << 16;
            if ((rc = alloc(&F_.type, nf_, err)) || (rc = alloc(&Fs_.type, nf_, err)) ||
                (rc = alloc(&zlist_, 2 * (size_t)zlist_cap_, err)) || (rc = alloc(&zcount_, 1, err)) ||
                (rc = alloc(&zlive_, id_cap_, err)) || (rc = alloc(&zcand_, id_cap_, err)))
                return rc;
        }
        if ((rc = alloc(&O_.r, nf_, err)) || (rc = alloc(&O_.v, nf_, err)) ||
            (rc = alloc(&O_.rho, nf_, err)) || (rc = alloc(&Br_, nf_, err)) ||
            (rc = alloc(&Bv_, nf_, err)) || (rc = alloc(&Brho_, nf_, err)) ||
            (rc = alloc(&keyB_, nf_, err)) || (rc = alloc(&slotB_, nf_, err)) ||
            (rc = alloc(&tmp_id_, nf_, err)) || (rc = alloc(&tmp_src_, nf_, err)) ||
            (rc = alloc(&perm_, nf_, err)) || (rc = alloc(&tmp_y_, nf_, err)))
            return rc;
        const int ntiles = (ncells_ + 1 + kScanTile - 1) / kScanTile;
        if (ntiles > kScanTile) {
            err = "grid too large for the scan";
            return 1;
        }
        if ((rc = alloc(&counts_, ncells_ + 1, err)) || (rc = alloc(&fstart_, ncells_ + 32, err)) ||
            (rc = alloc(&wstart_, ncells_ + 32, err)) || (rc = alloc(&tile_sums_, ntiles, err)) ||
            (rc = alloc(&health_, 1, err)) || (rc = alloc(&removed_, 1, err)) ||
            (rc = alloc(&rebuild_, 1, err)) || (rc = alloc(&body_runs_, 4, err)) ||
            (rc = alloc(&dtot_, 4 * (size_t)blocks_for(nf_), err)))
            return rc;
        if ((rc = alloc(&rm_cand_, id_cap_, err)) || (rc = alloc(&dead_, id_cap_, err)) ||
            (rc = alloc(&rm_list_, kRemovalCap, err)) || (rc = alloc(&rm_count_, 1, err)))
            return rc;
        TSPH_CK(cudaMemset(rm_cand_, 0, (size_t)std::max(id_cap_, 1)));
        TSPH_CK(cudaMemset(dead_, 0, (size_t)std::max(id_cap_, 1)));
        TSPH_CK(cudaMemset(rm_count_, 0, 4));
        TSPH_CK(cudaMemset(health_, 0, 4));
        TSPH_CK(cudaMemset(removed_, 0, 4));
        TSPH_CK(cudaMemset(body_runs_, 0, 16));
        TSPH_CK(cudaMemset(counts_, 0, sizeof(uint32_t) * (ncells_ + 1)));
        // staging
        if ((rc = alloc(&S_.r, id_cap_, err)) || (rc = alloc(&S_.v, id_cap_, err)) ||
            (rc = alloc(&S_.a, id_cap_, err)) || (rc = alloc(&S_.rho, id_cap_, err)) ||
            (rc = alloc(&S_.drho, id_cap_, err)) || (rc = alloc(&S_.p, id_cap_, err)) ||
            (rc = alloc(&S_.alive, id_cap_, err)))
            return rc;
        if (zones_on_ && (rc = alloc(&S_.type, id_cap_, err))) return rc;
        // ---- fluid initial state in index order
        {
            std::vector<double2> r(nf_, make_double2(0., 0.));
            std::vector<T2> v(nf_), a(nf_);
            std::vector<T> rho(nf_, T(0)), zero(nf_, T(0)), p(nf_, T(0));
            std::vector<uint32_t> id(nf_, 0u), key(nf_, 0u);
            std::vector<float2> loc(nf_, make_float2(0.f, 0.f));
            std::vector<uint8_t> typ(nf_, 0);
            for (int k = 0; k < nf0; k++) {
                const int i = fl[k];
                r[k] = make_double2(hs.r[2 * i], hs.r[2 * i + 1]);
                v[k].x = (T)hs.v[2 * i];
                v[k].y = (T)hs.v[2 * i + 1];
                a[k].x = (T)hs.a[2 * i];
                a[k].y = (T)hs.a[2 * i + 1];
                rho[k] = rho_stored_from_full<T>(hs.rho[i], hs.rho0);
                zero[k] = (T)hs.drho[i];
                p[k] = (T)hs.p[i];
                id[k] = (uint32_t)i;
                typ[k] = (uint8_t)hs.type[i];
            }
            if (zones_on_)
                TSPH_CK(cudaMemcpy(F_.type, typ.data(), (size_t)nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.r, r.data(), 16 * (size_t)nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.v, v.data(), sizeof(T2) * nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.a, a.data(), sizeof(T2) * nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.rho, rho.data(), sizeof(T) * nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.drho, zero.data(), sizeof(T) * nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.p, p.data(), sizeof(T) * nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.id, id.data(), 4 * (size_t)nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.key, key.data(), 4 * (size_t)nf_, cudaMemcpyHostToDevice));
            TSPH_CK(cudaMemcpy(F_.loc, loc.data(), 8 * (size_t)nf_, cudaMemcpyHostToDevice));
            // all entries live, none binned yet
            std::vector<uint32_t> fs(ncells_ + 2, 0u);
            fs[ncells_] = (uint32_t)nf0;
            fs[ncells_ + 1] = (uint32_t)nf0;
            TSPH_CK(cudaMemcpy(fstart_, fs.data(), 4 * fs.size(), cudaMemcpyHostToDevice));
        }
        // ---- walls: binned once on the host, sorted by (cell, index)
        {
            auto cell_of = [&](double x, const std::vector<long long> &b) -> int {
                const long long o = ordered_bits(x);
                if (o < b.front()) return -1;
                if (o >= b.back()) return (int)b.size() - 1;
                return (int)(std::upper_bound(b.begin(), b.end(), o) - b.begin()) - 1;
            };
            std::vector<std::pair<uint32_t, int>> order;
            for (int i : wl) {
                const int cx = cell_of(hs.r[2 * i], hs.bx), cy = cell_of(hs.r[2 * i + 1], hs.by);
                if (cx < 0 || cy < 0 || cx >= hs.ncx || cy >= hs.ncy) {
                    err = "wall particle " + std::to_string(i) + " lies outside the cell grid";
                    return 1;
                }
                order.push_back({(uint32_t)(cy + cx * hs.ncy), i});
            }
            if constexpr (std::is_same<T, float>::value) {
                std::sort(order.begin(), order.end(), [&](const std::pair<uint32_t, int> &a,
                                                          const std::pair<uint32_t, int> &b) {
                    if (a.first != b.first) return a.first < b.first;
                    const double ya = hs.r[2 * a.second + 1], yb = hs.r[2 * b.second + 1];
                    if (ya != yb) return ya < yb;
                    return a.second < b.second;
                });
            } else {
                std::sort(order.begin(), order.end());
            }
            if ((rc = alloc(&W_.r, nw_, err)) || (rc = alloc(&W_.loc, nw_, err)) ||
                (rc = alloc(&W_.key, nw_, err)) || (rc = alloc(&W_.id, nw_, err)) ||
                (rc = alloc(&W_.rho, nw_, err)) || (rc = alloc(&W_.drho, nw_, err)) ||
                (rc = alloc(&W_.p, nw_, err)) || (rc = alloc(&W_.rho_o, nw_, err)) ||
                (rc = alloc(&W_.gnr, nw_, err)) || (rc = alloc(&W_.gkey, nw_, err)) ||
                (rc = alloc(&W_.gloc, nw_, err)) || (rc = alloc(&W_.gnd, nw_, err)) ||
                (rc = alloc(&wall_zero_v_, nw_, err)))
                return rc;
            TSPH_CK(cudaMemset(wall_zero_v_, 0, sizeof(T2) * std::max(nw_, 1)));
            std::vector<double2> r(nw_), g(nw_);
            std::vector<float2> loc(nw_), gloc(nw_);
            std::vector<uint32_t> key(nw_), id(nw_), gkey(nw_);
            std::vector<T> rho(nw_), zero(nw_, T(0)), p(nw_);
            std::vector<T2> gnd(nw_);
            std::vector<uint32_t> ws(ncells_ + 1, 0u);
            for (int k = 0; k < nw_; k++) {
                const int i = order[k].second;
                const uint32_t c = order[k].first;
                const int cx = (int)(c / hs.ncy), cy = (int)(c % hs.ncy);
                const double x = hs.r[2 * i], y = hs.r[2 * i + 1];
                r[k] = make_double2(x, y);
                key[k] = c;
                id[k] = (uint32_t)i;
                loc[k] = make_float2((float)(x - hs.ox[cx]), (float)(y - hs.oy[cy]));
                rho[k] = rho_stored_from_full<T>(hs.rho[i], hs.rho0);
                zero[k] = (T)hs.drho[i];
                p[k] = (T)hs.p[i];
                ws[c + 1]++;
                const double gx = hs.has_gnr[i] ? hs.gnr[2 * i] : x;
                const double gy = hs.has_gnr[i] ? hs.gnr[2 * i + 1] : y;
                g[k] = make_double2(gx, gy);
                const int gcx = cell_of(gx, hs.bx), gcy = cell_of(gy, hs.by);
                if (gcx < 0 || gcy < 0 || gcx >= hs.ncx || gcy >= hs.ncy || !hs.has_gnr[i]) {
                    gkey[k] = (uint32_t)ncells_;
                    gloc[k] = make_float2(0.f, 0.f);
                } else {
                    gkey[k] = (uint32_t)(gcy + gcx * hs.ncy);
                    gloc[k] = make_float2((float)(gx - hs.ox[gcx]), (float)(gy - hs.oy[gcy]));
                }
                gnd[k].x = (T)(x - gx);
                gnd[k].y = (T)(y - gy);
            }
            for (int c = 0; c < ncells_; c++) ws[c + 1] += ws[c];
            if (nw_ > 0) {
                TSPH_CK(cudaMemcpy(W_.r, r.data(), 16 * (size_t)nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.loc, loc.data(), 8 * (size_t)nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.key, key.data(), 4 * (size_t)nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.id, id.data(), 4 * (size_t)nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.rho, rho.data(), sizeof(T) * nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.rho_o, rho.data(), sizeof(T) * nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.drho, zero.data(), sizeof(T) * nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.p, p.data(), sizeof(T) * nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.gnr, g.data(), 16 * (size_t)nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.gkey, gkey.data(), 4 * (size_t)nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.gloc, gloc.data(), 8 * (size_t)nw_, cudaMemcpyHostToDevice));
                TSPH_CK(cudaMemcpy(W_.gnd, gnd.data(), sizeof(T2) * nw_, cudaMemcpyHostToDevice));
            }
            TSPH_CK(cudaMemcpy(wstart_, ws.data(), 4 * ws.size(), cudaMemcpyHostToDevice));
        }
        TSPH_CK(cudaDeviceSynchronize());
        cells_ = false;
        return 0;
    }

    bool cells_valid() const override { return cells_; }
    void invalidate_cells() override { cells_ = false; }

    int particle_to_cell(std::string &err) override { return bin_particles(err, true); }

    // Particle_To_Cell.  With `allow_keep`, on a system whose fused step keeps
    // its cells (the pair-record step) and was binned before, the state (an
    // upload applied in the kept order) keeps its cells and lists when every
    // particle is still within sigma of where it was binned, as a step would:
    // the re-binning below then runs gated on the device flag that the check
    // sets (no host round trip), and the cells count as kept (calls that need
    // exact cells re-bin first).  Without it (exact cells asked for), the
    // state is re-binned.
    int bin_particles(std::string &err, bool allow_keep) {
        TSPH_FRESH_P(err);
        int rc;
        const uint32_t *gate = nullptr;
        bool kept = false;
        if constexpr (std::is_same<T, float>::value)
            if (allow_keep && binned_ && rec_f_.e && tile_shape_ == 2 && skin_ > 0.f &&
                wall_model_ != 2 && !zones_on_) {
                if ((rc = apply_staged_upload(err))) return rc;
                TSPH_CK(cudaMemsetAsync(pc_gate_, 0, 4, st_));
                if ((rc = launch(CAT_OTHER, k_upload_keep, blocks_for(nw_ + nf_), kBlock, err, F_,
                                 (const uint32_t *)fstart_, W_, nw_, grid_, P_,
                                 (const float2 *)lbin_, sig2_, (const uint32_t *)gen_, rec_f_,
                                 rec_w_, pc_gate_)))
                    return rc;
                gate = pc_gate_;
                kept = true;
            }
        if ((rc = apply_staged_upload(err))) return rc;
        if ((rc = zero_counts(err))) return rc;
        const int *nptr = reinterpret_cast<const int *>(fstart_ + ncells_);
        if ((rc = launch(CAT_SORT, k_bin_keep_dead, blocks_for(nf_), kBlock, err,
                         (const double2 *)F_.r, (const uint32_t *)F_.key, nptr, grid_, keyB_, slotB_,
                         counts_, health_, gate)))
            return rc;
        // gather everything into Fs_ (+ old state into B), then copy back
        if ((rc = sort_finish(F_.r, F_.v, F_.rho, F_.id, F_.a, F_.drho, F_.p, Fs_, O_.r, O_.v,
                              O_.rho, OldState<T>{Br_, Bv_, Brho_}, err, gate, F_.type)))
            return rc;
        if ((rc = launch(CAT_SORT, k_copy_state<T>, blocks_for(nf_), kBlock, err, F_,
                         (const FluidState<T>)Fs_, O_, OldState<T>{Br_, Bv_, Brho_},
                         (const uint32_t *)fstart_, ncells_, gate)))
            return rc;
        if (kept) {
            // the records and window table of the new order when it was
            // re-binned; its lists are then stale (a sort bumped the count),
            // and the first pass of the next step builds them
            if ((rc = pair_records(F_, gate, false, err))) return rc;
            cells_ = true;
            cells_kept_ = true;  // kept, or re-binned: settled when exact cells are asked for
            exported_ = false;
            return collect_profile(err);
        }
        // pair records and window table of the new order (FP32 build); with
        // kept lists (the fused step over pair records) also the lists of
        // the new order, built at the binned positions, so that the next
        // step keeps these cells
        if ((rc = pair_records(F_, nullptr, false, err))) return rc;
        if ((rc = build_lists(err))) return rc;
        cells_ = true;
        cells_kept_ = false;
        binned_ = true;
        exported_ = false;
        return collect_profile(err);
    }

    int density_to_pressure(std::string &err) override {
        int rc = launch(CAT_OTHER, k_eos<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                        (const uint32_t *)fstart_, ncells_, W_, nw_, P_, health_);
        if (rc) return rc;
        p_stale_ = false;
        return collect_profile(err);
    }

    int bt_density(std::string &err) override {
        TSPH_FRESH_P(err);
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        int rc = do_bt_density(err);
        if (rc) return rc;
        return collect_profile(err);
    }

    int mdbc_density(std::string &err) override {
        TSPH_FRESH_P(err);
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        int rc = do_mdbc(err);
        if (rc) return rc;
        return collect_profile(err);
    }

    int compute_forces(int model, std::string &err) override {
        TSPH_FRESH_P(err);
        if (cases_on_) {
            err = "packed cases: per-case gravity and removal boxes are applied by tsph_step only";
            return 8;
        }
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        int rc;
        if ((rc = ensure_exact_cells(err))) return rc;
        wall_model_ = model;
        if ((rc = fluid_pairs<MODE_FORCES>(F_, true, T(0), PairOut{}, err))) return rc;
        if (model == 1 && nw_ > 0 &&
            (rc = launch(CAT_OTHER, k_wall_rows<T>, blocks_for(nw_), kBlock, err, W_, nw_,
                         (const uint32_t *)fstart_, nbr_fluid(F_, true), grid_, P_, true, false, T(0),
                         (int32_t *)nullptr, (long long *)nullptr, (int32_t *)nullptr,
                         (const uint32_t *)nullptr, false, PairRec{})))
            return rc;
        return collect_profile(err);
    }

    int predictor(double dt, std::string &err) override {
        TSPH_FRESH_P(err);
        int rc = launch(CAT_OTHER, k_predict_inplace<T>, blocks_for(nw_ + nf_), kBlock, err, F_, O_,
                        (const uint32_t *)fstart_, ncells_, W_, nw_, (T)dt);
        if (rc) return rc;
        cells_ = false;
        return collect_profile(err);
    }

    int corrector(double dt, std::string &err) override {
        TSPH_FRESH_P(err);
        if (cases_on_) {
            err = "packed cases: per-case gravity and removal boxes are applied by tsph_step only";
            return 8;
        }
        int rc = launch(CAT_OTHER, k_correct_inplace<T>, blocks_for(nw_ + nf_), kBlock, err, F_, O_,
                        (const uint32_t *)fstart_, ncells_, W_, nw_, (T)dt, P_.rho0);
        if (rc) return rc;
        cells_ = false;
        return collect_profile(err);
    }

    // RemoveParticlesOutOfDomain with the reference's skip of the particle
    // after an erased one (the fused step's corrector removes every particle
    // outside the box instead)
    int remove_out_of_domain(int *removed, std::string &err) override {
        TSPH_FRESH_P(err);
        if (cases_on_) {
            err = "packed cases: per-case gravity and removal boxes are applied by tsph_step only";
            return 8;
        }
        int rc;
        if (!zlive_ && ((rc = alloc(&zlive_, id_cap_, err)) || (rc = alloc(&zcand_, id_cap_, err))))
            return rc;
        TSPH_CK(cudaMemsetAsync(removed_, 0, 4, st_));
        TSPH_CK(cudaMemsetAsync(zlive_, 0, (size_t)ntot_, st_));
        TSPH_CK(cudaMemsetAsync(zcand_, 0, (size_t)ntot_, st_));
        if ((rc = launch(CAT_OTHER, k_remove_mark<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, (const uint32_t *)W_.id, nw_, box_,
                         zlive_, zcand_)) ||
            (rc = launch(CAT_OTHER, k_remove_apply<T>, blocks_for(nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, (const uint8_t *)zlive_,
                         (const uint8_t *)zcand_, removed_, health_, dead_)))
            return rc;
        uint32_t h = 0;
        TSPH_CK(cudaMemcpyAsync(&h, removed_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        if (removed) *removed = (int)h;
        if (h) cells_ = false;
        return collect_profile(err);
    }

    // the RUN body of a case with buffer zones (cases/inflowSlab_mDBC/
    // SPH_simulationSymplectic.h): the per-function sequence with every
    // zone's inlet or outlet after the predictor
    int step_zones(int model, double dt, std::string &err) {
        int rc;
        wall_model_ = model;
        if (model == 0 && (rc = do_mdbc(err))) return rc;
        if (model == 2 && (rc = do_bt_density(err))) return rc;
        if ((rc = density_to_pressure(err)) || (rc = predictor(dt, err))) return rc;
        for (int z = 0; z < (int)zones_.size(); z++) {
            const int t = zones_[z].btype;
            if ((rc = (t >= 11 ? bz_outlet(z, dt, err) : bz_inlet(z, dt, err)))) return rc;
        }
        int removed = 0;
        if ((rc = particle_to_cell(err)) || (rc = density_to_pressure(err)) ||
            (rc = compute_forces(model, err)) || (rc = corrector(dt, err)) ||
            (rc = remove_out_of_domain(&removed, err)) || (rc = particle_to_cell(err)) ||
            (rc = density_to_pressure(err)) || (rc = compute_forces(model, err)))
            return rc;
        return 0;
    }

    int step(int model, double dt, int nsteps, std::string &err) override {
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        if (cases_on_ && model != 0) {
            err = "packed cases: mDBC walls only";
            return 8;
        }
        int rc;
        if (zones_on_) {
            for (int s = 0; s < nsteps; s++)
                if ((rc = step_zones(model, dt, err))) return rc;
            exported_ = false;
            return 0;
        }
        wall_model_ = model;
        if (tile_shape_ < 0 && (rc = autotune(nullptr, nullptr, err))) return rc;
        if (prof_) {
            for (int s = 0; s < nsteps; s++)
                if ((rc = enqueue_step(model, (T)dt, err))) return rc;
        } else {
            long long bits;
            std::memcpy(&bits, &dt, 8);
            auto key = std::make_pair(model, bits);
            auto it = graphs_.find(key);
            if (it == graphs_.end()) {
                cudaGraph_t g;
                TSPH_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
                capturing_ = true;
                cap_main_ = 0;
                for (int b = 0; b < 4; b++) cap_body_[b] = 0;
                rc = enqueue_step(model, (T)dt, err);
                capturing_ = false;
                cudaGraph_t g2 = nullptr;
                cudaError_t e = cudaStreamEndCapture(st_, &g2);
                if (rc) {
                    if (g2) cudaGraphDestroy(g2);
                    return rc;
                }
                if (e != cudaSuccess) {
                    err = std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e);
                    return 2;
                }
                g = g2;
                cudaGraphExec_t ex;
                e = cudaGraphInstantiate(&ex, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e);
                    return 2;
                }
                it = graphs_.emplace(key, ex).first;
                graph_kernels_[key] = cap_main_;
                for (int b = 1; b < 4; b++)
                    if (cap_body_[b]) body_kernels_[b] = cap_body_[b];
            }
            for (int s = 0; s < nsteps; s++) TSPH_CK(cudaGraphLaunch(it->second, st_));
            launched_ += (long long)nsteps * graph_kernels_[key];
        }
        // the reference's state after a step holds p = EOS(rho) (step body
        // :110-111): formed by the next entry point that reads the state
        p_stale_ = true;
        cells_ = true;
        // with kept lists the cells are those of the last binning, which may
        // be some steps old (every particle within sigma of where it was binned)
        if constexpr (std::is_same<T, float>::value)
            if (skin_ > 0.f && tile_shape_ == 2 && model != 2 && !zones_on_) {
                cells_kept_ = true;
                rec_passes_ += nsteps;  // graph replays run kept-list passes too
            }
        exported_ = false;
        return collect_profile(err);
    }

    int kernel_launches(long long *count, int reset, std::string &err) override {
        (void)err;
        uint32_t runs[4] = {0, 0, 0, 0};
        TSPH_CK(cudaMemcpyAsync(runs, body_runs_, 16, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        *count = launched_;
        for (int b = 1; b < 4; b++) *count += (long long)runs[b] * body_kernels_[b];
        if (reset) {
            launched_ = 0;
            TSPH_CK(cudaMemsetAsync(body_runs_, 0, 16, st_));
        }
        return 0;
    }

    int np_live(int *np, std::string &err) override {
        uint32_t nl = 0, rm = 0;
        TSPH_CK(cudaMemcpyAsync(&nl, fstart_ + ncells_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        // particles marked by tsph_remove_out_of_domain but not yet re-binned
        if (!cells_ok()) {
            std::vector<uint32_t> key(nl);
            if (nl) TSPH_CK(cudaMemcpy(key.data(), F_.key, 4 * (size_t)nl, cudaMemcpyDeviceToHost));
            for (uint32_t k : key) rm += (k == (uint32_t)ncells_);
        }
        *np = (int)(nl - rm) + nw_;
        return 0;
    }

    // after k_export: whether every particle is alive (counted on the device),
    // and the alive map on the host only when some are not
    uint32_t *alive_count_ = nullptr;
    // Without buffer zones the index space is fixed and walls are never
    // removed, so every index is live exactly when the live fluid count plus
    // the walls equals the index count: one 4-byte read.  The count is that of
    // the last binning, so it is used only while the cells are fresh (a
    // removal marks particles dead and leaves the cells stale until the next
    // binning); otherwise dense stays false and the alive map decides.
    int dense_by_count(bool &dense, std::string &err) {
        (void)err;
        dense = false;
        if (zones_on_ || !cells_) return 0;
        uint32_t nl = 0;
        TSPH_CK(cudaMemcpyAsync(&nl, fstart_ + ncells_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        dense = (long long)nl + nw_ == (long long)ntot_;
        return 0;
    }

    // after k_export wrote S_.alive: whether every index is live, else the map
    int alive_map(std::vector<uint8_t> &alive, bool &dense, std::string &err) {
        int rc;
        if (!zones_on_ && cells_) {
            if ((rc = dense_by_count(dense, err))) return rc;
            if (!dense) {
                alive.resize(ntot_);
                TSPH_CK(cudaMemcpyAsync(alive.data(), S_.alive, ntot_, cudaMemcpyDeviceToHost, st_));
                TSPH_CK(cudaStreamSynchronize(st_));
            }
            return 0;
        }
        if (!alive_count_ && (rc = alloc(&alive_count_, 1, err))) return rc;
        TSPH_CK(cudaMemsetAsync(alive_count_, 0, 4, st_));
        if ((rc = launch(CAT_OTHER, k_count_alive,
                         std::min(blocks_for((long long)(ntot_ >> 2) + 1), 4 * 152), kBlock, err,
                         (const uint8_t *)S_.alive, ntot_, alive_count_)))
            return rc;
        uint32_t cnt = 0;
        TSPH_CK(cudaMemcpyAsync(&cnt, alive_count_, 4, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        dense = cnt == (uint32_t)ntot_;
        if (!dense) {
            alive.resize(ntot_);
            TSPH_CK(cudaMemcpyAsync(alive.data(), S_.alive, ntot_, cudaMemcpyDeviceToHost, st_));
            TSPH_CK(cudaStreamSynchronize(st_));
        }
        return 0;
    }

    int download(int mask, double *r, double *v, double *a, double *rho, double *drho, double *p,
                 int32_t *index, int32_t *type, std::string &err) override {
        // the stored pressure is brought up to date only when it is asked for
        if (mask & kFieldP) TSPH_FRESH_P(err);
        if (up_pending_) {  // its staging set holds the staged upload
            err = "an upload is staged: call tsph_particle_to_cell first";
            return 3;
        }
        TSPH_CK(cudaMemsetAsync(S_.alive, 0, ntot_, st_));
        int rc = launch(CAT_OTHER, k_export<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                        (const uint32_t *)fstart_, ncells_, W_, nw_, P_.rho0, S_, mask & 63);
        if (rc) return rc;
        std::vector<uint8_t> alive;
        bool dense = false;
        if ((rc = alive_map(alive, dense, err))) return rc;
        std::vector<double> tmp;
        auto fetch = [&](int bit, const void *src, double *dst, int width) -> int {
            if (!(mask & bit) || !dst) return 0;
            if (dense) {
                TSPH_CK(cudaMemcpyAsync(dst, src, 8 * (size_t)width * ntot_, cudaMemcpyDeviceToHost, st_));
                return 0;
            }
            tmp.resize((size_t)width * ntot_);
            TSPH_CK(cudaMemcpyAsync(tmp.data(), src, 8 * (size_t)width * ntot_, cudaMemcpyDeviceToHost, st_));
            TSPH_CK(cudaStreamSynchronize(st_));
            size_t o = 0;
            for (int i = 0; i < ntot_; i++)
                if (alive[i]) {
                    for (int w = 0; w < width; w++) dst[o * width + w] = tmp[(size_t)i * width + w];
                    o++;
                }
            return 0;
        };
        if ((rc = fetch(1, S_.r, r, 2)) || (rc = fetch(2, S_.v, v, 2)) || (rc = fetch(4, S_.a, a, 2)) ||
            (rc = fetch(8, S_.rho, rho, 1)) || (rc = fetch(16, S_.drho, drho, 1)) ||
            (rc = fetch(32, S_.p, p, 1)))
            return rc;
        TSPH_CK(cudaStreamSynchronize(st_));
        if ((mask & 64) && index) {
            int o = 0;
            for (int i = 0; i < ntot_; i++)
                if (dense || alive[i]) index[o++] = i;
        }
        if (type && S_.type) {  // buffer zones change types: read them from the device
            std::vector<int32_t> t(ntot_);
            TSPH_CK(cudaMemcpyAsync(t.data(), S_.type, 4 * (size_t)ntot_, cudaMemcpyDeviceToHost, st_));
            TSPH_CK(cudaStreamSynchronize(st_));
            int o = 0;
            for (int i = 0; i < ntot_; i++)
                if (dense || alive[i]) type[o++] = t[i];
        }
        return collect_profile(err);
    }

    // tsph_download_async: the export into a staging set of its own on the
    // system's stream, then the device-to-host copies on a copy stream, so
    // that the copies run beside whatever the caller enqueues next (the next
    // step's upload and kernels); download_wait ends them.  One download in
    // flight at a time.  States with erased particles take the synchronous
    // path (their rows are compacted on the host).
    int download_async(int mask, double *r, double *v, double *a, double *rho, double *drho,
                       double *p, std::string &err) override {
        if (mask & kFieldP) TSPH_FRESH_P(err);
        int rc;
        if (mask & ~63) {
            err = "tsph_download_async: r, v, a, rho, drho and p only";
            return 1;
        }
        if ((rc = download_wait(err))) return rc;
        bool dense = false;
        if ((rc = dense_by_count(dense, err))) return rc;
        if (!dense) return download(mask, r, v, a, rho, drho, p, nullptr, nullptr, err);
        if (!D_.r) {
            if ((rc = alloc(&D_.r, id_cap_, err)) || (rc = alloc(&D_.v, id_cap_, err)) ||
                (rc = alloc(&D_.a, id_cap_, err)) || (rc = alloc(&D_.rho, id_cap_, err)) ||
                (rc = alloc(&D_.drho, id_cap_, err)) || (rc = alloc(&D_.p, id_cap_, err)) ||
                (rc = alloc(&D_.alive, id_cap_, err)))
                return rc;
            TSPH_CK(cudaStreamCreateWithFlags(&cs_, cudaStreamNonBlocking));
            TSPH_CK(cudaEventCreateWithFlags(&ev_x_, cudaEventDisableTiming));
            TSPH_CK(cudaEventCreateWithFlags(&ev_d_, cudaEventDisableTiming));
        }
        if ((rc = launch(CAT_OTHER, k_export<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, W_, nw_, P_.rho0, D_, mask)))
            return rc;
        TSPH_CK(cudaEventRecord(ev_x_, st_));
        TSPH_CK(cudaStreamWaitEvent(cs_, ev_x_, 0));
        const void *src[6] = {D_.r, D_.v, D_.a, D_.rho, D_.drho, D_.p};
        double *dst[6] = {r, v, a, rho, drho, p};
        for (int k = 0; k < 6; k++)
            if ((mask & (1 << k)) && dst[k])
                TSPH_CK(cudaMemcpyAsync(dst[k], src[k], (k < 3 ? 16 : 8) * (size_t)ntot_,
                                        cudaMemcpyDeviceToHost, cs_));
        TSPH_CK(cudaEventRecord(ev_d_, cs_));
        d_pending_ = true;
        return 0;
    }

    int download_wait(std::string &err) override {
        if (!d_pending_) return 0;
        d_pending_ = false;
        TSPH_CK(cudaEventSynchronize(ev_d_));
        return 0;
    }

    int upload_async(int mask, const double *r, const double *v, const double *a,
                     const double *rho, const double *drho, const double *p,
                     std::string &err) override {
        // (only stages copies: the pressure is brought up to date by the
        // tsph_particle_to_cell that applies them, before it does)
        if (mask & ~63) {
            err = "tsph_upload_async: r, v, a, rho, drho and p only";
            return 1;
        }
        if (zones_on_) {
            err = "tsph_upload_async: systems with buffer zones use tsph_upload";
            return 8;
        }
        if (up_pending_) {
            err = "an upload is staged: call tsph_particle_to_cell first";
            return 3;
        }
        if (!cu_) {
            TSPH_CK(cudaStreamCreateWithFlags(&cu_, cudaStreamNonBlocking));
            TSPH_CK(cudaEventCreateWithFlags(&ev_up_, cudaEventDisableTiming));
            TSPH_CK(cudaEventCreateWithFlags(&ev_imp_, cudaEventDisableTiming));
            TSPH_CK(cudaEventRecord(ev_imp_, st_));
        }
        // the staging set is free once the last staged import has read it
        TSPH_CK(cudaStreamWaitEvent(cu_, ev_imp_, 0));
        void *dst[6] = {S_.r, S_.v, S_.a, S_.rho, S_.drho, S_.p};
        const double *src[6] = {r, v, a, rho, drho, p};
        int m = 0;
        for (int k = 0; k < 6; k++)
            if ((mask & (1 << k)) && src[k]) {
                TSPH_CK(cudaMemcpyAsync(dst[k], src[k], (k < 3 ? 16 : 8) * (size_t)ntot_,
                                        cudaMemcpyHostToDevice, cu_));
                m |= 1 << k;
            }
        TSPH_CK(cudaEventRecord(ev_up_, cu_));
        up_pending_ = true;
        up_mask_ = m;
        return 0;
    }

    // cell lists valid and no staged upload waiting for particle_to_cell
    bool cells_ok() const { return cells_ && !up_pending_; }

    // the staged upload into the state (start of particle_to_cell)
    int apply_staged_upload(std::string &err) {
        if (!up_pending_) return 0;
        up_pending_ = false;
        TSPH_CK(cudaStreamWaitEvent(st_, ev_up_, 0));
        int rc = launch(CAT_OTHER, k_import<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                        (const uint32_t *)fstart_, ncells_, W_, nw_, P_.rho0, S_, up_mask_,
                        ntot_, health_);
        if (rc) return rc;
        TSPH_CK(cudaEventRecord(ev_imp_, st_));
        return 0;
    }

    int upload(int mask, const double *r, const double *v, const double *a, const double *rho,
               const double *drho, const double *p, std::string &err) override {
        TSPH_FRESH_P(err);
        if (up_pending_) {
            err = "an upload is staged: call tsph_particle_to_cell first";
            return 3;
        }
        // every index live (the usual case) needs no alive map
        int rc;
        std::vector<uint8_t> alive;
        bool dense = false;
        if ((rc = dense_by_count(dense, err))) return rc;
        if (!dense) {
            // alive map from the device
            TSPH_CK(cudaMemsetAsync(S_.alive, 0, ntot_, st_));
            rc = launch(CAT_OTHER, k_export<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                        (const uint32_t *)fstart_, ncells_, W_, nw_, P_.rho0, S_, 0);
            if (rc) return rc;
            if ((rc = alive_map(alive, dense, err))) return rc;
        }
        std::vector<double> tmp;
        auto put = [&](int bit, void *dst, const double *src, int width) -> int {
            if (!(mask & bit) || !src) return 0;
            if (dense) {
                TSPH_CK(cudaMemcpyAsync(dst, src, 8 * (size_t)width * ntot_, cudaMemcpyHostToDevice, st_));
                return 0;
            }
            tmp.assign((size_t)width * ntot_, 0.0);
            size_t o = 0;
            for (int i = 0; i < ntot_; i++)
                if (alive[i]) {
                    for (int w = 0; w < width; w++) tmp[(size_t)i * width + w] = src[o * width + w];
                    o++;
                }
            TSPH_CK(cudaMemcpyAsync(dst, tmp.data(), 8 * (size_t)width * ntot_, cudaMemcpyHostToDevice, st_));
            TSPH_CK(cudaStreamSynchronize(st_));
            return 0;
        };
        if ((rc = put(1, S_.r, r, 2)) || (rc = put(2, S_.v, v, 2)) || (rc = put(4, S_.a, a, 2)) ||
            (rc = put(8, S_.rho, rho, 1)) || (rc = put(16, S_.drho, drho, 1)) ||
            (rc = put(32, S_.p, p, 1)))
            return rc;
        // walls keep r and v (static); only fluid rows take them
        if ((rc = launch(CAT_OTHER, k_import<T>, blocks_for(nw_ + nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, ncells_, W_, nw_, P_.rho0, S_, mask & 63, -1,
                         health_)))
            return rc;
        TSPH_CK(cudaStreamSynchronize(st_));
        if (mask & 1) cells_ = false;
        return collect_profile(err);
    }

    int get_cells(int32_t *cell_start, int32_t *cell_list, std::string &err) override {
        TSPH_FRESH_P(err);
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        int rc0;
        if ((rc0 = ensure_exact_cells(err))) return rc0;
        TSPH_CK(cudaStreamSynchronize(st_));
        std::vector<uint32_t> fs(ncells_ + 2), ws(ncells_ + 1), fid(nf_), wid(nw_);
        TSPH_CK(cudaMemcpy(fs.data(), fstart_, 4 * fs.size(), cudaMemcpyDeviceToHost));
        TSPH_CK(cudaMemcpy(ws.data(), wstart_, 4 * ws.size(), cudaMemcpyDeviceToHost));
        if (nf_) TSPH_CK(cudaMemcpy(fid.data(), F_.id, 4 * (size_t)nf_, cudaMemcpyDeviceToHost));
        if (nw_) TSPH_CK(cudaMemcpy(wid.data(), W_.id, 4 * (size_t)nw_, cudaMemcpyDeviceToHost));
        // reference numbering: rank of the original index among live particles
        std::vector<int> alive(ntot_, 0);
        for (int c = 0; c < ncells_; c++)
            for (uint32_t j = fs[c]; j < fs[c + 1]; j++) alive[fid[j]] = 1;
        for (int w = 0; w < nw_; w++) alive[wid[w]] = 1;
        std::vector<int> rank(ntot_, -1);
        int o = 0;
        for (int i = 0; i < ntot_; i++)
            if (alive[i]) rank[i] = o++;
        int acc = 0;
        std::vector<int> tmp;
        for (int c = 0; c < ncells_; c++) {
            cell_start[c] = acc;
            tmp.clear();
            for (uint32_t j = ws[c]; j < ws[c + 1]; j++) tmp.push_back(rank[wid[j]]);
            for (uint32_t j = fs[c]; j < fs[c + 1]; j++) tmp.push_back(rank[fid[j]]);
            std::sort(tmp.begin(), tmp.end());
            for (int x : tmp) cell_list[acc++] = x;
        }
        cell_start[ncells_] = acc;
        return 0;
    }

    int pair_digest(int32_t *count, int64_t *sum, int32_t *xr, std::string &err) override {
        TSPH_FRESH_P(err);
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        int rc0;
        if ((rc0 = ensure_exact_cells(err))) return rc0;
        int rc;
        if (!dig_count_) {
            if ((rc = alloc(&dig_count_, id_cap_, err)) || (rc = alloc(&dig_sum_, id_cap_, err)) ||
                (rc = alloc(&dig_xor_, id_cap_, err)))
                return rc;
        }
        // fluid rows into [0, nf), wall rows into [nf, nf + nw)
        if ((rc = launch(CAT_OTHER, k_fluid_pairs<T, MODE_DIGEST>, blocks_for(nf_), kBlock, err, F_,
                         (const uint32_t *)fstart_, (const uint32_t *)wstart_, nbr_fluid(F_, true),
                         nbr_walls(true), grid_, P_, O_, T(0), PairOut{}, health_, dig_count_,
                         dig_sum_, dig_xor_, (const uint32_t *)W_.id)))
            return rc;
        if (nw_ &&
            (rc = launch(CAT_OTHER, k_wall_rows<T>, blocks_for(nw_), kBlock, err, W_, nw_,
                         (const uint32_t *)fstart_, nbr_fluid(F_, true), grid_, P_, true, false, T(0),
                         dig_count_ + nf_, dig_sum_ + nf_, dig_xor_ + nf_, (const uint32_t *)F_.id,
                         true, PairRec{})))
            return rc;
        TSPH_CK(cudaStreamSynchronize(st_));
        uint32_t nl = 0;
        TSPH_CK(cudaMemcpy(&nl, fstart_ + ncells_, 4, cudaMemcpyDeviceToHost));
        std::vector<int32_t> c(nl + nw_), x(nl + nw_);
        std::vector<long long> s(nl + nw_);
        std::vector<uint32_t> fid(nl), wid(nw_);
        if (nl) {
            TSPH_CK(cudaMemcpy(c.data(), dig_count_, 4 * (size_t)nl, cudaMemcpyDeviceToHost));
            TSPH_CK(cudaMemcpy(s.data(), dig_sum_, 8 * (size_t)nl, cudaMemcpyDeviceToHost));
            TSPH_CK(cudaMemcpy(x.data(), dig_xor_, 4 * (size_t)nl, cudaMemcpyDeviceToHost));
            TSPH_CK(cudaMemcpy(fid.data(), F_.id, 4 * (size_t)nl, cudaMemcpyDeviceToHost));
        }
        if (nw_) {
            TSPH_CK(cudaMemcpy(c.data() + nl, dig_count_ + nf_, 4 * (size_t)nw_, cudaMemcpyDeviceToHost));
            TSPH_CK(cudaMemcpy(s.data() + nl, dig_sum_ + nf_, 8 * (size_t)nw_, cudaMemcpyDeviceToHost));
            TSPH_CK(cudaMemcpy(x.data() + nl, dig_xor_ + nf_, 4 * (size_t)nw_, cudaMemcpyDeviceToHost));
            TSPH_CK(cudaMemcpy(wid.data(), W_.id, 4 * (size_t)nw_, cudaMemcpyDeviceToHost));
        }
        // rows in ascending original index
        std::vector<std::pair<uint32_t, int>> rows;
        for (uint32_t j = 0; j < nl; j++) rows.push_back({fid[j], (int)j});
        for (int w = 0; w < nw_; w++) rows.push_back({wid[w], (int)nl + w});
        std::sort(rows.begin(), rows.end());
        for (size_t k = 0; k < rows.size(); k++) {
            count[k] = c[rows[k].second];
            sum[k] = s[rows[k].second];
            xr[k] = x[rows[k].second];
        }
        return 0;
    }

    int health(uint32_t *flags, int clear, std::string &err) override {
        TSPH_CK(cudaMemcpyAsync(flags, health_, 4, cudaMemcpyDeviceToHost, st_));
        if (clear) TSPH_CK(cudaMemsetAsync(health_, 0, 4, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        return 0;
    }

    int totals(double out[4], std::string &err) override {
        TSPH_FRESH_P(err);
        const int nb = blocks_for(nf_);
        int rc = launch(CAT_OTHER, k_totals<T>, nb, kBlock, err, F_, (const uint32_t *)fstart_,
                        ncells_, m64_, dtot_);
        if (rc) return rc;
        std::vector<double> h(4 * (size_t)nb);
        TSPH_CK(cudaMemcpyAsync(h.data(), dtot_, 8 * h.size(), cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        for (int q = 0; q < 4; q++) out[q] = 0;
        for (int b = 0; b < nb; b++)
            for (int q = 0; q < 4; q++) out[q] += h[(size_t)b * 4 + q];
        return collect_profile(err);
    }

    ProbeSrc<T> probe_src() const {
        constexpr bool shifted = std::is_same<T, float>::value;
        return ProbeSrc<T>{F_.r, F_.v, F_.rho, F_.p, W_.r, W_.rho, W_.p,
                           (const uint32_t *)fstart_, (const uint32_t *)wstart_, grid_, P_.hd,
                           (double)P_.awen, (double)P_.bwen, m64_, shifted ? (double)P_.rho0 : 0.0};
    }

    // device scratch for the probes, `bytes` at least
    int probe_scratch(size_t bytes, std::string &err) {
        if (bytes <= pr_cap_) return 0;
        if (pr_d_) cudaFree(pr_d_);
        pr_d_ = nullptr;
        pr_cap_ = 0;
        TSPH_CK(cudaMalloc(&pr_d_, bytes));
        pr_cap_ = bytes;
        return 0;
    }

    int water_level(int n, const double *x, const double *y0, const int32_t *inverse, double *out,
                    std::string &err) override {
        TSPH_FRESH_P(err);
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        // the sample heights of each gauge, accumulated as the reference does
        // (ar.y += i dp_wl, src/SPH_water_level.h:96-101); past the grid the
        // kernel volume is 0, so the sequence ends there
        const double dp_wl = dp64_ * 0.00005;
        const int nmax = (int)(box_.ym / dp_wl);
        const double top = box_.ym + 2.0 * (double)P_.kh, bot = box_.y0 - 2.0 * (double)P_.kh;
        std::vector<double> ys;
        std::vector<int> off(n + 1, 0), inv(n);
        for (int g = 0; g < n; g++) {
            off[g] = (int)ys.size();
            inv[g] = inverse && inverse[g] ? 1 : 0;
            double ay = y0[g];
            for (int i = 0; i < nmax; i++) {
                if (inv[g]) ay -= i * dp_wl;
                else ay += i * dp_wl;
                ys.push_back(ay);
                if (inv[g] ? ay < bot : ay > top) break;
            }
        }
        off[n] = (int)ys.size();
        const size_t nb = 8 * ys.size() + 8 * (size_t)n + 4 * (size_t)(n + 1) + 4 * (size_t)n * 2 + 64;
        int rc;
        if ((rc = probe_scratch(nb, err))) return rc;
        double *d_ys = pr_d_;
        double *d_x = d_ys + ys.size();
        int *d_off = reinterpret_cast<int *>(d_x + n);
        int *d_inv = d_off + n + 1;
        int *d_first = d_inv + n;
        TSPH_CK(cudaMemcpyAsync(d_ys, ys.data(), 8 * ys.size(), cudaMemcpyHostToDevice, st_));
        TSPH_CK(cudaMemcpyAsync(d_x, x, 8 * (size_t)n, cudaMemcpyHostToDevice, st_));
        TSPH_CK(cudaMemcpyAsync(d_off, off.data(), 4 * (size_t)(n + 1), cudaMemcpyHostToDevice, st_));
        TSPH_CK(cudaMemcpyAsync(d_inv, inv.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, st_));
        int most = 1;
        for (int g = 0; g < n; g++) most = std::max(most, off[g + 1] - off[g]);
        TSPH_CK(cudaMemsetAsync(d_first, 0x7f, 4 * (size_t)n, st_));
        const dim3 wl_grid((unsigned)n, (unsigned)((most + kWlChunk - 1) / kWlChunk));
        k_water_level<T><<<wl_grid, 256, 0, st_>>>(probe_src(), (const double *)d_x,
                                                   (const int *)d_inv, (const double *)d_ys,
                                                   (const int *)d_off, d_first);
        TSPH_CK(cudaGetLastError());
        std::vector<int> first(n);
        TSPH_CK(cudaMemcpyAsync(first.data(), d_first, 4 * (size_t)n, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        for (int g = 0; g < n; g++) {
            const int i = first[g];
            if (i < 0 || i >= off[g + 1] - off[g]) {
                out[g] = std::nan("");
                continue;
            }
            const double ay = ys[(size_t)off[g] + i];
            out[g] = inv[g] ? ay + i * dp_wl : ay - i * dp_wl;
        }
        return collect_profile(err);
    }

    int point_fields(int n, const double *xy, double *out, std::string &err) override {
        TSPH_FRESH_P(err);
        if (!cells_ok()) {
            err = "cell lists are stale: call tsph_particle_to_cell first";
            return 3;
        }
        int rc;
        if ((rc = probe_scratch(8 * 6 * (size_t)n + 64, err))) return rc;
        double *d_xy = pr_d_, *d_out = pr_d_ + 2 * (size_t)n;
        TSPH_CK(cudaMemcpyAsync(d_xy, xy, 16 * (size_t)n, cudaMemcpyHostToDevice, st_));
        if ((rc = launch(CAT_OTHER, k_point_fields<T>, (int)(((long long)n * 32 + 255) / 256), 256,
                         err, probe_src(), (const double *)d_xy, n, d_out)))
            return rc;
        TSPH_CK(cudaMemcpyAsync(out, d_out, 32 * (size_t)n, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        return collect_profile(err);
    }

    int water_front(double y_max, double *x, std::string &err) override {
        TSPH_FRESH_P(err);
        int rc;
        if ((rc = probe_scratch(64, err))) return rc;
        unsigned long long *d_best = reinterpret_cast<unsigned long long *>(pr_d_);
        TSPH_CK(cudaMemsetAsync(d_best, 0, 8, st_));
        if ((rc = launch(CAT_OTHER, k_water_front, blocks_for(nf_), kBlock, err, (const double2 *)F_.r,
                         (const uint32_t *)fstart_, ncells_, y_max, d_best)))
            return rc;
        unsigned long long best = 0;
        TSPH_CK(cudaMemcpyAsync(&best, d_best, 8, cudaMemcpyDeviceToHost, st_));
        TSPH_CK(cudaStreamSynchronize(st_));
        *x = best ? from_ordered((long long)(best ^ 0x8000000000000000ULL)) : std::nan("");
        return collect_profile(err);
    }

    int sync(std::string &err) override {
        TSPH_CK(cudaStreamSynchronize(st_));
        return collect_profile(err);
    }

    void set_profiling(bool on) override { prof_ = on; }
    Profile profile(bool reset) override {
        Profile p = acc_;
        if (reset) acc_ = Profile{};
        return p;
    }
};

}  // namespace tsph
