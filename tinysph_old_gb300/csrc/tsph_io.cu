// tsph_io.cu -- host-side output and checkpoint of a system: the reference's
// ASCII VTK snapshot (write_to_ASCII_VTK, src/SPH_data_to_vtk.h:4-51) and a
// binary checkpoint that restarts a run where it stopped.
#include <cstdint>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/tsph.h"
#include "tsph_system.h"

namespace {

int io_fail(int code, const std::string &m) {
    tsph::set_last_error(m);
    return code;
}

struct Snapshot {
    std::vector<double> r, v, a, rho, drho, p;
    std::vector<int32_t> index, type;
    int n = 0;
};

int snapshot(tsph_system *s, Snapshot &z) {
    int rc = tsph_np(s, &z.n);
    if (rc) return rc;
    const int n = z.n;
    z.r.resize(2 * (size_t)n);
    z.v.resize(2 * (size_t)n);
    z.a.resize(2 * (size_t)n);
    z.rho.resize(n);
    z.drho.resize(n);
    z.p.resize(n);
    z.index.resize(n);
    z.type.resize(n);
    tsph_host_state hs = {z.r.data(), z.v.data(), z.a.data(), z.rho.data(),
                          z.drho.data(), z.p.data(), z.index.data(), z.type.data()};
    return tsph_download(s, TSPH_F_R | TSPH_F_V | TSPH_F_A | TSPH_F_RHO | TSPH_F_DRHO | TSPH_F_P |
                                TSPH_F_INDEX | TSPH_F_TYPE,
                         &hs);
}

const char kMagic[8] = {'T', 'S', 'P', 'H', 'C', 'K', 'P', '1'};

template <typename T> void put(std::ofstream &f, const T *p, size_t n) {
    f.write(reinterpret_cast<const char *>(p), (std::streamsize)(sizeof(T) * n));
}
template <typename T> bool get(std::ifstream &f, T *p, size_t n) {
    f.read(reinterpret_cast<char *>(p), (std::streamsize)(sizeof(T) * n));
    return (bool)f;
}

}  // namespace

extern "C" {

int tsph_write_vtk(tsph_system *s, const char *path) {
    if (!s || !path) return io_fail(TSPH_ERR_ARG, "null argument");
    Snapshot z;
    int rc = snapshot(s, z);
    if (rc) return rc;
    std::ofstream file(path);
    if (!file) return io_fail(TSPH_ERR_ARG, std::string("cannot open ") + path);
    const int np = z.n;
    // the layout and the stream formatting of write_to_ASCII_VTK
    file << "# vtk DataFile Version 3.0" << std::endl << "vtk output" << std::endl << "ASCII"
         << std::endl << "DATASET POLYDATA" << std::endl;
    file << "POINTS " << np << " float" << std::endl;
    for (int i = 0; i < np; i++) file << z.r[2 * i] << " " << z.r[2 * i + 1] << " 0" << std::endl;
    file << "POINT_DATA " << np << std::endl << "FIELDS FieldData 4" << std::endl;
    file << "type 1 " << np << " int" << std::endl;
    for (int i = 0; i < np; i++) file << z.type[i] << std::endl;
    file << "pressure 1 " << np << " float" << std::endl;
    for (int i = 0; i < np; i++) file << z.p[i] << std::endl;
    file << "density 1 " << np << " float" << std::endl;
    for (int i = 0; i < np; i++) file << z.rho[i] << std::endl;
    file << "velocity 3 " << np << " float" << std::endl;
    for (int i = 0; i < np; i++) file << z.v[2 * i] << " " << z.v[2 * i + 1] << " 0" << std::endl;
    if (!file) return io_fail(TSPH_ERR_ARG, std::string("write failed: ") + path);
    return TSPH_OK;
}

int tsph_save_checkpoint(tsph_system *s, const char *path) {
    if (!s || !path) return io_fail(TSPH_ERR_ARG, "null argument");
    if (!s->hs.case_g.empty())
        return io_fail(TSPH_ERR_UNSUPPORTED, "checkpoints of packed cases are not written");
    // a system stepping with kept neighbour lists is re-binned first, so the
    // run that goes on and a run restarted from the file continue from the
    // same binning (and so bit for bit alike)
    if (s->eng) {
        std::string err;
        if (s->eng->settle_cells(err)) return io_fail(TSPH_ERR_CUDA, err);
    }
    Snapshot z;
    int rc = snapshot(s, z);
    if (rc) return rc;
    const tsph::HostSetup &hs = s->hs;
    const int n = z.n;
    std::vector<double> gnr(2 * (size_t)n, 0.0);
    std::vector<uint8_t> has(n, 0);
    for (int k = 0; k < n; k++) {
        // particles an inlet appended have indices past the ones given at
        // setup, and no ghost node
        const size_t i = (size_t)z.index[k];
        if (i >= hs.has_gnr.size()) continue;
        gnr[2 * k] = hs.gnr[2 * i];
        gnr[2 * k + 1] = hs.gnr[2 * i + 1];
        has[k] = hs.has_gnr[i];
    }
    std::ofstream f(path, std::ios::binary);
    if (!f) return io_fail(TSPH_ERR_ARG, std::string("cannot open ") + path);
    // version 2: version 1 followed by the buffer zones and their capacities
    const int32_t head[4] = {2, s->precision, s->eng ? s->eng->tile_shape() : -1, n};
    const int32_t nz = (int32_t)(hs.zones.size() / 12);
    const int32_t zcap[2] = {hs.extra_rows, hs.extra_ids};
    const double cst[11] = {hs.h, hs.kap, hs.cs, hs.rho0, hs.visco, hs.delta, hs.dp,
                            hs.x0, hs.xm, hs.y0, hs.ym};
    f.write(kMagic, 8);
    put(f, head, 4);
    put(f, cst, 11);
    put(f, z.type.data(), n);
    put(f, z.r.data(), 2 * (size_t)n);
    put(f, z.v.data(), 2 * (size_t)n);
    put(f, z.a.data(), 2 * (size_t)n);
    put(f, z.rho.data(), n);
    put(f, z.drho.data(), n);
    put(f, z.p.data(), n);
    put(f, gnr.data(), 2 * (size_t)n);
    put(f, has.data(), n);
    put(f, &nz, 1);
    put(f, hs.zones.data(), hs.zones.size());
    put(f, zcap, 2);
    if (!f) return io_fail(TSPH_ERR_ARG, std::string("write failed: ") + path);
    return TSPH_OK;
}

int tsph_load_checkpoint(const char *path, void *stream, tsph_system **out) {
    if (!path || !out) return io_fail(TSPH_ERR_ARG, "null argument");
    *out = nullptr;
    std::ifstream f(path, std::ios::binary);
    if (!f) return io_fail(TSPH_ERR_ARG, std::string("cannot open ") + path);
    char magic[8];
    int32_t head[4];
    double cst[11];
    if (!get(f, magic, 8) || std::memcmp(magic, kMagic, 8) != 0 || !get(f, head, 4) ||
        (head[0] != 1 && head[0] != 2) || head[3] < 0 || !get(f, cst, 11))
        return io_fail(TSPH_ERR_ARG, std::string("not a checkpoint of this library: ") + path);
    const int n = head[3];
    std::vector<int32_t> type(n);
    std::vector<double> r(2 * (size_t)n), v(2 * (size_t)n), a(2 * (size_t)n), rho(n), drho(n),
        p(n), gnr(2 * (size_t)n);
    std::vector<uint8_t> has(n);
    if (!get(f, type.data(), n) || !get(f, r.data(), 2 * (size_t)n) ||
        !get(f, v.data(), 2 * (size_t)n) || !get(f, a.data(), 2 * (size_t)n) ||
        !get(f, rho.data(), n) || !get(f, drho.data(), n) || !get(f, p.data(), n) ||
        !get(f, gnr.data(), 2 * (size_t)n) || !get(f, has.data(), n))
        return io_fail(TSPH_ERR_ARG, std::string("truncated checkpoint: ") + path);
    int32_t nz = 0, zcap[2] = {0, 0};
    std::vector<double> zones;
    if (head[0] >= 2) {
        if (!get(f, &nz, 1) || nz < 0 || nz > 4096)
            return io_fail(TSPH_ERR_ARG, std::string("truncated checkpoint: ") + path);
        zones.resize(12 * (size_t)nz);
        if (!get(f, zones.data(), zones.size()) || !get(f, zcap, 2))
            return io_fail(TSPH_ERR_ARG, std::string("truncated checkpoint: ") + path);
    }
    bool any_gnr = false;
    for (int k = 0; k < n; k++) any_gnr |= has[k] != 0;
    const tsph_constants c = {cst[0], cst[1], cst[2], cst[3], cst[4], cst[5], cst[6]};
    const tsph_domain d = {cst[7], cst[8], cst[9], cst[10]};
    tsph_system *s = nullptr;
    int rc = tsph_create(&c, &d, head[1], stream, &s);
    if (rc) return rc;
    // zones as tsph_add_buffer_zone stores them: ox, oy, x0, y0, xm, ym, nbl,
    // b_len, b_height, btype, vx, vy
    for (int32_t k = 0; k < nz && !rc; k++) {
        const double *q = &zones[12 * (size_t)k];
        rc = tsph_add_buffer_zone(s, q[2], q[4], q[3], q[5], (int)q[6], q[10], q[11], q[0], q[1],
                                  (int)q[9]);
    }
    if (!rc && nz > 0) rc = tsph_set_zone_capacity(s, zcap[0], zcap[1]);
    if (rc) {
        tsph_destroy(s);
        return rc;
    }
    // the saved variant of the pair kernel before the binning, which then
    // prepares what that variant keeps (neighbour lists)
    if ((rc = tsph_add_particles(s, n, type.data(), r.data(), v.data(), rho.data(), p.data(),
                                 any_gnr ? gnr.data() : nullptr)) ||
        (rc = tsph_divide_to_cells(s)) ||
        (head[2] >= 0 && (rc = tsph_set_tile_shape(s, head[2]))) ||
        (rc = tsph_particle_to_cell(s))) {
        tsph_destroy(s);
        return rc;
    }
    tsph_host_state in = {nullptr, nullptr, a.data(), nullptr, drho.data(), nullptr, nullptr,
                          nullptr};
    if ((rc = tsph_upload(s, TSPH_F_A | TSPH_F_DRHO, &in))) {
        tsph_destroy(s);
        return rc;
    }
    *out = s;
    return TSPH_OK;
}

}  // extern "C"
