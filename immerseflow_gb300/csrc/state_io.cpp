// state_io.cpp -- checkpoint / restart and time-history output.
//
// Restart: the reference parses `Restart Restart_Time` (src/main.cu:27-30) and
// `Write Interval` (src/main.cu:50-53) but uses neither; its Fortran
// predecessor restarts from an ASCII snapshot Data/data.NNNNNNN.dat (three
// header lines, then one row per cell, j outer and i inner: x y u v p and three
// more columns; test/UTIL_PRE_SIM.f90:120-149).  Two forms here:
//  * binary checkpoint: every array a METHOD-mode step carries into the next
//    (cell and face velocities, convection history, pressure, outflow boundary
//    values, the per-instance iteration state), so that a run restarted from it
//    continues bit for bit; checked by a header (grid size, grid and body
//    hash, payload hash).  REFERENCE mode keeps u, v, p.
//  * ASCII snapshot in the predecessor's layout, the three extra columns being
//    uf (east face), vf (north face) and iblank.  It holds no convection
//    history, so the first step after an ASCII restart starts Adams-Bashforth
//    again with a forward-Euler convection step, like the first step of a run.
//
// Time history: the predecessor's probe_init (test/UTIL_PRE_SIM.f90:172-202)
// reads probe.dat (count, a skipped line, one "x y" per probe), takes the
// nearest cell centre in x and in y (first minimum of |x - x_probe|), and
// writes probe_output.dat (a header with the count, locations and indices, a
// blank line, "Time  U   V  P", then one row per step).  Here the step's last
// kernel appends a record (step, cd, cl, u, v, p at each probe cell) to a
// device ring buffer, so recording costs no host synchronisation.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "ifx_host.h"

using namespace ifx;

namespace {

#define SIO_CUDA(x)                                                                      \
    do {                                                                                 \
        cudaError_t e_ = (x);                                                            \
        if (e_ != cudaSuccess)                                                           \
            return set_error(IFX_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define SIO_TRY(x)                   \
    do {                             \
        ifx_status s_ = (x);         \
        if (s_ != IFX_OK) return s_; \
    } while (0)

constexpr char kMagic[8] = {'I', 'F', 'X', 'C', 'K', 'P', 'T', '1'};
constexpr char kSetMagic[8] = {'I', 'F', 'X', 'C', 'K', 'S', 'E', 'T'};
// 2: the pressures of the two steps before (initial-guess extrapolation);
// 3: the predictor increment of the step before (the predictor's initial guess)
constexpr uint32_t kVersion = 3;

struct CkptHeader {
    char magic[8];
    uint32_t version, header_bytes;
    int32_t mode, precision, NX, NY;
    int32_t qstride, state_bytes;
    int64_t steps;
    double dt, re;
    uint64_t geom_hash;
    uint64_t payload_bytes;
    uint64_t payload_hash;
};
static_assert(sizeof(CkptHeader) % 8 == 0, "checkpoint header packing");

// FNV-1a, 64 bit.
uint64_t fnv1a(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t k = 0; k < n; k++) {
        h ^= b[k];
        h *= 1099511628211ull;
    }
    return h;
}

// Grid faces, body and boundary types: what the state's meaning depends on.
uint64_t geom_hash(const Instance& I) {
    uint64_t h = fnv1a(I.xf.data(), I.xf.size() * sizeof(double));
    h = fnv1a(I.yf.data(), I.yf.size() * sizeof(double), h);
    const ifx_config& c = I.cfg;
    const double body[5] = {c.body_cx, c.body_cy, c.body_a, c.body_b, c.body_angle_deg};
    h = fnv1a(&c.body, sizeof(c.body), h);
    if (c.body) h = fnv1a(body, sizeof(body), h);
    h = fnv1a(c.bc_type, sizeof(c.bc_type), h);
    return h;
}

bool method(const ifx_solver* S) { return S->mode == IFX_MODE_METHOD; }

size_t cells(const Instance& I) { return (size_t)I.nx * I.ny; }

// Cell fields a METHOD-mode checkpoint carries: u, v, U, V, the convection
// history Nu, Nv, p, the pressures of the two steps before and the predictor
// increment of the step before.
constexpr int kMethodFields = 11;

size_t payload_bytes(const ifx_solver* S, const Instance& I) {
    if (!method(S)) return 3 * cells(I) * sizeof(double);
    return kMethodFields * cells(I) * sizeof(double) + 2 * 4 * (size_t)I.qstride * sizeof(double) + sizeof(InstState);
}

// Pitched device field <-> dense host rows.
ifx_status field_out(ifx_solver* S, const Instance& I, const double* dev, size_t pitch, double* host) {
    SIO_CUDA(cudaMemcpy2DAsync(host, I.nx * 8, dev, pitch * 8, I.nx * 8, I.ny, cudaMemcpyDeviceToHost, S->stream));
    return IFX_OK;
}
ifx_status field_in(ifx_solver* S, const Instance& I, double* dev, size_t pitch, const double* host) {
    SIO_CUDA(cudaMemcpy2DAsync(dev, pitch * 8, host, I.nx * 8, I.nx * 8, I.ny, cudaMemcpyHostToDevice, S->stream));
    return IFX_OK;
}

ifx_status check_inst(const ifx_solver* S, int inst, const char* fn) {
    if (!S || inst < 0 || inst >= (int)S->inst.size()) return set_error(IFX_ERR_ARG, std::string(fn) + ": bad argument");
    return IFX_OK;
}
// The same for saving or restoring a state: the geometry of a moving body
// (cell types, ghost slots, stencil bytes of every level) is not part of it.
ifx_status check_restartable(const ifx_solver* S, int inst, const char* fn) {
    SIO_TRY(check_inst(S, inst, fn));
    if (S->inst[inst].moving)
        return set_error(IFX_ERR_STATE, std::string(fn) + ": not supported for a moving body's instance");
    return IFX_OK;
}

// The METHOD-mode cell arrays of a checkpoint, in order.
void method_fields(const InstDev& d, double* (&f)[kMethodFields]) {
    f[0] = d.u; f[1] = d.v; f[2] = d.U; f[3] = d.V; f[4] = d.Nu; f[5] = d.Nv; f[6] = d.p; f[7] = d.pold;
    f[8] = d.pold2; f[9] = d.dup; f[10] = d.dvp;
}

// REFERENCE-mode arrays (dense rows).
void reference_fields(ifx_solver* S, double* (&f)[3]) {
    f[0] = S->r_cur ? S->r_ut : S->r_u;
    f[1] = S->r_cur ? S->r_vt : S->r_v;
    f[2] = S->r_p;
}

// Outflow face values from the cell next to each outflow ghost, as at creation.
ifx_status rebuild_outflow(ifx_solver* S, const Instance& I, const std::vector<double>& u, const std::vector<double>& v) {
    if (I.ghost_cnt == 0) return IFX_OK;
    std::vector<GhostDev> g(I.ghost_cnt);
    SIO_CUDA(cudaMemcpyAsync(g.data(), S->dG + I.ghost_beg, g.size() * sizeof(GhostDev), cudaMemcpyDeviceToHost, S->stream));
    SIO_CUDA(cudaStreamSynchronize(S->stream));
    std::vector<double> qbu(4 * (size_t)I.qstride, 0.0), qbv(4 * (size_t)I.qstride, 0.0);
    auto dense = [&](int c) { return (size_t)(c % I.pitch) + (size_t)(c / I.pitch) * I.nx; };
    for (const GhostDev& e : g)
        if (e.qown >= 0) {
            qbu[e.qown] = u[dense(e.adj)];
            qbv[e.qown] = v[dense(e.adj)];
        }
    SIO_CUDA(cudaMemcpyAsync(I.dev.qbu, qbu.data(), qbu.size() * 8, cudaMemcpyHostToDevice, S->stream));
    SIO_CUDA(cudaMemcpyAsync(I.dev.qbv, qbv.data(), qbv.size() * 8, cudaMemcpyHostToDevice, S->stream));
    SIO_CUDA(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

bool write_file(const std::string& path, const std::vector<char>& data) {
    const std::string tmp = path + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
    if (std::fclose(f) != 0 || !ok) {
        std::remove(tmp.c_str());
        return false;
    }
    return std::rename(tmp.c_str(), path.c_str()) == 0;
}

bool read_file(const std::string& path, std::vector<char>& data) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    data.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return true;
}

}  // namespace

// ------------------------------------------------------------ checkpoints

extern "C" ifx_status ifx_checkpoint_bytes(const ifx_solver* S, int inst, size_t* bytes) {
    SIO_TRY(check_restartable(S, inst, "ifx_checkpoint_bytes"));
    if (!bytes) return set_error(IFX_ERR_ARG, "ifx_checkpoint_bytes: bad argument");
    *bytes = sizeof(CkptHeader) + payload_bytes(S, S->inst[inst]);
    return IFX_OK;
}

extern "C" ifx_status ifx_checkpoint_save(ifx_solver* S, int inst, void* buf, size_t n) {
    SIO_TRY(check_restartable(S, inst, "ifx_checkpoint_save"));
    size_t need = 0;
    SIO_TRY(ifx_checkpoint_bytes(S, inst, &need));
    if (!buf || n < need) return set_error(IFX_ERR_ARG, "ifx_checkpoint_save: buffer smaller than ifx_checkpoint_bytes");
    SIO_CUDA(cudaSetDevice(S->device));
    SIO_TRY(finish_pending(S));
    const Instance& I = S->inst[inst];
    CkptHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.header_bytes = sizeof(CkptHeader);
    h.mode = S->mode;
    h.precision = S->prec;
    h.NX = I.NX;
    h.NY = I.NY;
    h.qstride = I.qstride;
    h.state_bytes = method(S) ? (int32_t)sizeof(InstState) : 0;
    h.dt = I.cfg.dt;
    h.re = I.cfg.re;
    h.geom_hash = geom_hash(I);
    h.payload_bytes = payload_bytes(S, I);
    char* pay = (char*)buf + sizeof(CkptHeader);
    double* q = (double*)pay;
    const size_t nc = cells(I);
    if (method(S)) {
        double* f[kMethodFields];
        method_fields(I.dev, f);
        for (int k = 0; k < kMethodFields; k++) SIO_TRY(field_out(S, I, f[k], I.pitch, q + k * nc));
        double* qb = q + kMethodFields * nc;
        SIO_CUDA(cudaMemcpyAsync(qb, I.dev.qbu, 4 * (size_t)I.qstride * 8, cudaMemcpyDeviceToHost, S->stream));
        SIO_CUDA(cudaMemcpyAsync(qb + 4 * (size_t)I.qstride, I.dev.qbv, 4 * (size_t)I.qstride * 8, cudaMemcpyDeviceToHost,
                                 S->stream));
        InstState st;
        SIO_CUDA(cudaMemcpyAsync(&st, S->dS + inst, sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
        SIO_CUDA(cudaStreamSynchronize(S->stream));
        std::memcpy(qb + 8 * (size_t)I.qstride, &st, sizeof(InstState));
        h.steps = st.nstep;
    } else {
        double* f[3];
        reference_fields(S, f);
        for (int k = 0; k < 3; k++) SIO_TRY(field_out(S, I, f[k], I.nx, q + k * nc));
        SIO_CUDA(cudaStreamSynchronize(S->stream));
        h.steps = S->steps_done;
    }
    h.payload_hash = fnv1a(pay, h.payload_bytes);
    std::memcpy(buf, &h, sizeof(h));
    return IFX_OK;
}

namespace {

// Every check of a checkpoint record against instance inst (header, format,
// mode, grid and geometry hash, sizes, payload checksum), on the host only:
// nothing on the device changes until a record has passed.
ifx_status validate_checkpoint(const ifx_solver* S, int inst, const void* buf, size_t n, CkptHeader* out) {
    if (!buf || n < sizeof(CkptHeader)) return set_error(IFX_ERR_PARSE, "ifx_checkpoint_load: not a checkpoint (too short)");
    CkptHeader h;
    std::memcpy(&h, buf, sizeof(h));
    const Instance& I = S->inst[inst];
    if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion || h.header_bytes != sizeof(CkptHeader))
        return set_error(IFX_ERR_PARSE, "ifx_checkpoint_load: not a checkpoint of this format");
    if (h.mode != S->mode) return set_error(IFX_ERR_ARG, "ifx_checkpoint_load: checkpoint of the other solver mode");
    if (h.NX != I.NX || h.NY != I.NY || h.qstride != I.qstride || h.geom_hash != geom_hash(I))
        return set_error(IFX_ERR_ARG, "ifx_checkpoint_load: checkpoint of a different grid, body or boundary set-up");
    if (h.state_bytes != (method(S) ? (int32_t)sizeof(InstState) : 0) || h.payload_bytes != payload_bytes(S, I) ||
        n < sizeof(CkptHeader) + h.payload_bytes)
        return set_error(IFX_ERR_PARSE, "ifx_checkpoint_load: truncated or mismatched checkpoint");
    const char* pay = (const char*)buf + sizeof(CkptHeader);
    if (fnv1a(pay, h.payload_bytes) != h.payload_hash) return set_error(IFX_ERR_PARSE, "ifx_checkpoint_load: checksum mismatch");
    if (out) *out = h;
    return IFX_OK;
}

}  // namespace

extern "C" ifx_status ifx_checkpoint_load(ifx_solver* S, int inst, const void* buf, size_t n) {
    SIO_TRY(check_restartable(S, inst, "ifx_checkpoint_load"));
    CkptHeader h;
    SIO_TRY(validate_checkpoint(S, inst, buf, n, &h));
    const Instance& I = S->inst[inst];
    const char* pay = (const char*)buf + sizeof(CkptHeader);
    SIO_CUDA(cudaSetDevice(S->device));
    SIO_TRY(finish_pending(S));
    // aligned copy of the payload (the caller's buffer may be unaligned)
    std::vector<double> q((h.payload_bytes + 7) / 8);
    std::memcpy(q.data(), pay, h.payload_bytes);
    const size_t nc = cells(I);
    if (method(S)) {
        double* f[kMethodFields];
        method_fields(I.dev, f);
        for (int k = 0; k < kMethodFields; k++) SIO_TRY(field_in(S, I, f[k], I.pitch, q.data() + k * nc));
        // Jacobi partners start equal to the state, as at creation
        SIO_TRY(field_in(S, I, I.dev.u2, I.pitch, q.data()));
        SIO_TRY(field_in(S, I, I.dev.v2, I.pitch, q.data() + nc));
        const double* qb = q.data() + kMethodFields * nc;
        SIO_CUDA(cudaMemcpyAsync(I.dev.qbu, qb, 4 * (size_t)I.qstride * 8, cudaMemcpyHostToDevice, S->stream));
        SIO_CUDA(cudaMemcpyAsync(I.dev.qbv, qb + 4 * (size_t)I.qstride, 4 * (size_t)I.qstride * 8, cudaMemcpyHostToDevice,
                                 S->stream));
        InstState st;
        std::memcpy(&st, qb + 8 * (size_t)I.qstride, sizeof(InstState));
        InstState cur;
        SIO_CUDA(cudaMemcpyAsync(&cur, S->dS + inst, sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
        SIO_CUDA(cudaStreamSynchronize(S->stream));
        st.hist_n = cur.hist_n;  // the time history belongs to this handle
        SIO_CUDA(cudaMemcpyAsync(S->dS + inst, &st, sizeof(InstState), cudaMemcpyHostToDevice, S->stream));
    } else {
        double* f[3];
        reference_fields(S, f);
        for (int k = 0; k < 3; k++) SIO_TRY(field_in(S, I, f[k], I.nx, q.data() + k * nc));
    }
    SIO_CUDA(cudaStreamSynchronize(S->stream));
    if (S->inst.size() == 1) S->steps_done = h.steps;
    return IFX_OK;
}

extern "C" ifx_status ifx_checkpoint_write(ifx_solver* S, const char* path) {
    if (!S || !path) return set_error(IFX_ERR_ARG, "ifx_checkpoint_write: bad argument");
    std::vector<char> out(16);
    std::memcpy(out.data(), kSetMagic, 8);
    const uint32_t ver = kVersion, count = (uint32_t)S->inst.size();
    std::memcpy(out.data() + 8, &ver, 4);
    std::memcpy(out.data() + 12, &count, 4);
    for (int k = 0; k < (int)count; k++) {
        size_t nb = 0;
        SIO_TRY(ifx_checkpoint_bytes(S, k, &nb));
        const uint64_t n64 = nb;
        const size_t at = out.size();
        out.resize(at + 8 + nb);
        std::memcpy(out.data() + at, &n64, 8);
        SIO_TRY(ifx_checkpoint_save(S, k, out.data() + at + 8, nb));
    }
    if (!write_file(path, out)) return set_error(IFX_ERR_IO, std::string("ifx_checkpoint_write: cannot write ") + path);
    return IFX_OK;
}

extern "C" ifx_status ifx_checkpoint_read(ifx_solver* S, const char* path) {
    if (!S || !path) return set_error(IFX_ERR_ARG, "ifx_checkpoint_read: bad argument");
    std::vector<char> in;
    if (!read_file(path, in)) return set_error(IFX_ERR_IO, std::string("ifx_checkpoint_read: cannot read ") + path);
    uint32_t ver = 0, count = 0;
    if (in.size() < 16 || std::memcmp(in.data(), kSetMagic, 8) != 0)
        return set_error(IFX_ERR_PARSE, "ifx_checkpoint_read: not a checkpoint file");
    std::memcpy(&ver, in.data() + 8, 4);
    std::memcpy(&count, in.data() + 12, 4);
    if (ver != kVersion) return set_error(IFX_ERR_PARSE, "ifx_checkpoint_read: unknown checkpoint version");
    if (count != S->inst.size()) return set_error(IFX_ERR_ARG, "ifx_checkpoint_read: instance count differs");
    // every record is checked before any instance is loaded, so a file with a
    // bad record leaves the whole handle as it was
    std::vector<std::pair<size_t, size_t>> rec(count);
    size_t at = 16;
    for (int k = 0; k < (int)count; k++) {
        SIO_TRY(check_restartable(S, k, "ifx_checkpoint_read"));
        uint64_t nb = 0;
        if (at + 8 > in.size()) return set_error(IFX_ERR_PARSE, "ifx_checkpoint_read: truncated file");
        std::memcpy(&nb, in.data() + at, 8);
        at += 8;
        if (nb > in.size() - at) return set_error(IFX_ERR_PARSE, "ifx_checkpoint_read: truncated file");
        ifx_status st = validate_checkpoint(S, k, in.data() + at, (size_t)nb, nullptr);
        if (st != IFX_OK)
            return set_error(st, "ifx_checkpoint_read: record " + std::to_string(k) + ": " + ifx_last_error());
        rec[k] = {at, (size_t)nb};
        at += nb;
    }
    for (int k = 0; k < (int)count; k++) SIO_TRY(ifx_checkpoint_load(S, k, in.data() + rec[k].first, rec[k].second));
    return IFX_OK;
}

// ------------------------------------------------ ASCII snapshot (predecessor layout)

extern "C" ifx_status ifx_write_snapshot_ascii(ifx_solver* S, int inst, const char* path) {
    SIO_TRY(check_inst(S, inst, "ifx_write_snapshot_ascii"));
    if (!path) return set_error(IFX_ERR_ARG, "ifx_write_snapshot_ascii: bad argument");
    SIO_CUDA(cudaSetDevice(S->device));
    SIO_TRY(finish_pending(S));
    const Instance& I = S->inst[inst];
    const int nx = I.nx, ny = I.ny;
    const size_t nc = cells(I);
    std::vector<double> u(nc), v(nc), p(nc), uf(nc, 0.0), vf(nc, 0.0), ib(nc);
    long long steps = S->steps_done;
    SIO_TRY(ifx_get_field_i(S, inst, IFX_FIELD_U, u.data(), nc));
    SIO_TRY(ifx_get_field_i(S, inst, IFX_FIELD_V, v.data(), nc));
    SIO_TRY(ifx_get_field_i(S, inst, IFX_FIELD_P, p.data(), nc));
    SIO_TRY(ifx_get_field_i(S, inst, IFX_FIELD_IBLANK, ib.data(), nc));
    if (method(S)) {
        SIO_TRY(field_out(S, I, I.dev.U, I.pitch, uf.data()));
        SIO_TRY(field_out(S, I, I.dev.V, I.pitch, vf.data()));
        InstState st;
        SIO_CUDA(cudaMemcpyAsync(&st, S->dS + inst, sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
        SIO_CUDA(cudaStreamSynchronize(S->stream));
        steps = st.nstep;
    } else {
        std::vector<double> a((size_t)(nx - 1) * (ny - 2)), b((size_t)(nx - 2) * (ny - 1));
        SIO_TRY(ifx_get_field_i(S, inst, IFX_FIELD_UF, a.data(), a.size()));
        SIO_TRY(ifx_get_field_i(S, inst, IFX_FIELD_VF, b.data(), b.size()));
        for (int j = 1; j < ny - 1; j++)
            for (int i = 0; i < nx - 1; i++) uf[i + (size_t)j * nx] = a[i + (size_t)(j - 1) * (nx - 1)];
        for (int j = 0; j < ny - 1; j++)
            for (int i = 1; i < nx - 1; i++) vf[i + (size_t)j * nx] = b[(i - 1) + (size_t)j * (nx - 2)];
    }
    FILE* f = std::fopen(path, "w");
    if (!f) return set_error(IFX_ERR_IO, std::string("ifx_write_snapshot_ascii: cannot write ") + path);
    std::fprintf(f, "TITLE = \"ImmerseFlow restart snapshot\"\n");
    std::fprintf(f, "VARIABLES = \"X\",\"Y\",\"U\",\"V\",\"P\",\"UF\",\"VF\",\"IBLANK\"\n");
    std::fprintf(f, "ZONE T=\"step %lld\", I=%d, J=%d, DATAPACKING=POINT\n", steps, nx, ny);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            const size_t c = i + (size_t)j * nx;
            std::fprintf(f, "%.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", I.xc[i], I.yc[j], u[c], v[c], p[c], uf[c],
                         vf[c], ib[c]);
        }
    if (std::fclose(f) != 0) return set_error(IFX_ERR_IO, std::string("ifx_write_snapshot_ascii: cannot write ") + path);
    return IFX_OK;
}

extern "C" ifx_status ifx_read_snapshot_ascii(ifx_solver* S, int inst, const char* path) {
    SIO_TRY(check_restartable(S, inst, "ifx_read_snapshot_ascii"));
    if (!path) return set_error(IFX_ERR_ARG, "ifx_read_snapshot_ascii: bad argument");
    std::ifstream in(path);
    if (!in) return set_error(IFX_ERR_IO, std::string("ifx_read_snapshot_ascii: cannot read ") + path);
    const Instance& I = S->inst[inst];
    const int nx = I.nx, ny = I.ny;
    const size_t nc = cells(I);
    std::string line;
    long long steps = -1;
    for (int k = 0; k < 3; k++) {
        if (!std::getline(in, line)) return set_error(IFX_ERR_PARSE, "ifx_read_snapshot_ascii: missing header");
        const size_t at = line.find("step ");
        if (k == 2 && at != std::string::npos) steps = std::atoll(line.c_str() + at + 5);
    }
    std::vector<double> u(nc), v(nc), p(nc), uf(nc), vf(nc);
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
            if (!std::getline(in, line)) return set_error(IFX_ERR_PARSE, "ifx_read_snapshot_ascii: fewer rows than cells");
            for (char& ch : line)
                if (ch == ',') ch = ' ';
            std::istringstream row(line);
            double x, y, ib;
            const size_t c = i + (size_t)j * nx;
            if (!(row >> x >> y >> u[c] >> v[c] >> p[c] >> uf[c] >> vf[c] >> ib))
                return set_error(IFX_ERR_PARSE, "ifx_read_snapshot_ascii: row " + std::to_string(c + 4) + " needs 8 numbers");
            if (std::fabs(x - I.xc[i]) > 1e-9 * (1.0 + std::fabs(I.xc[i])) ||
                std::fabs(y - I.yc[j]) > 1e-9 * (1.0 + std::fabs(I.yc[j])))
                return set_error(IFX_ERR_ARG, "ifx_read_snapshot_ascii: cell centres differ from this grid");
        }
    SIO_CUDA(cudaSetDevice(S->device));
    SIO_TRY(finish_pending(S));
    if (method(S)) {
        const InstDev& d = I.dev;
        SIO_TRY(field_in(S, I, d.u, I.pitch, u.data()));
        SIO_TRY(field_in(S, I, d.v, I.pitch, v.data()));
        SIO_TRY(field_in(S, I, d.u2, I.pitch, u.data()));
        SIO_TRY(field_in(S, I, d.v2, I.pitch, v.data()));
        SIO_TRY(field_in(S, I, d.p, I.pitch, p.data()));
        SIO_TRY(field_in(S, I, d.U, I.pitch, uf.data()));
        SIO_TRY(field_in(S, I, d.V, I.pitch, vf.data()));
        SIO_TRY(rebuild_outflow(S, I, u, v));
        InstState st;
        SIO_CUDA(cudaMemcpyAsync(&st, S->dS + inst, sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
        SIO_CUDA(cudaStreamSynchronize(S->stream));
        st.have_nold = 0;  // no convection history in this format
        st.pold_n = 0;     // nor the pressures of the steps before
        // nor the predictor increment of the step before
        SIO_CUDA(cudaMemsetAsync(d.dup, 0, I.ncell * sizeof(double), S->stream));
        SIO_CUDA(cudaMemsetAsync(d.dvp, 0, I.ncell * sizeof(double), S->stream));
        if (steps >= 0) st.nstep = steps;
        SIO_CUDA(cudaMemcpyAsync(S->dS + inst, &st, sizeof(InstState), cudaMemcpyHostToDevice, S->stream));
    } else {
        double* f[3];
        reference_fields(S, f);
        SIO_TRY(field_in(S, I, f[0], I.nx, u.data()));
        SIO_TRY(field_in(S, I, f[1], I.nx, v.data()));
        SIO_TRY(field_in(S, I, f[2], I.nx, p.data()));
    }
    SIO_CUDA(cudaStreamSynchronize(S->stream));
    if (S->inst.size() == 1 && steps >= 0) S->steps_done = steps;
    return IFX_OK;
}

// ------------------------------------------------------------ time history

extern "C" ifx_status ifx_probes_read(const char* path, int cap, double* xy, int* n) {
    if (!path || !n || (cap > 0 && !xy)) return set_error(IFX_ERR_ARG, "ifx_probes_read: bad argument");
    std::ifstream in(path);
    if (!in) return set_error(IFX_ERR_IO, std::string("ifx_probes_read: cannot read ") + path);
    std::string line;
    int count = -1;
    if (!std::getline(in, line) || !(std::istringstream(line) >> count) || count < 0)
        return set_error(IFX_ERR_PARSE, "ifx_probes_read: first line must hold the probe count");
    std::getline(in, line);  // skipped, as in probe_init
    for (int k = 0; k < count; k++) {
        double x, y;
        if (!std::getline(in, line)) return set_error(IFX_ERR_PARSE, "ifx_probes_read: fewer probe lines than the count");
        for (char& ch : line)
            if (ch == ',') ch = ' ';
        if (!(std::istringstream(line) >> x >> y)) return set_error(IFX_ERR_PARSE, "ifx_probes_read: a probe line needs x y");
        if (k < cap) {
            xy[2 * k] = x;
            xy[2 * k + 1] = y;
        }
    }
    *n = count;
    return IFX_OK;
}

namespace {
// First index of the smallest |c[k] - x| (Fortran minloc).
int nearest(const std::vector<double>& c, double x) {
    int best = 0;
    for (int k = 1; k < (int)c.size(); k++)
        if (std::fabs(c[k] - x) < std::fabs(c[best] - x)) best = k;
    return best;
}

void free_tracked(ifx_solver* S, void* p) {
    if (!p) return;
    for (size_t k = 0; k < S->allocs.size(); k++)
        if (S->allocs[k] == p) {
            S->allocs.erase(S->allocs.begin() + k);
            break;
        }
    cudaFree(p);
}

ifx_status alloc_tracked(ifx_solver* S, void** p, size_t bytes) {
    SIO_CUDA(cudaMalloc(p, bytes));
    S->allocs.push_back(*p);
    S->device_bytes += bytes;
    return IFX_OK;
}
}  // namespace

extern "C" ifx_status ifx_set_history(ifx_solver* S, int inst, int capacity, int nprobes, const double* xy) {
    SIO_TRY(check_inst(S, inst, "ifx_set_history"));
    if (capacity < 0 || nprobes < 0 || (nprobes > 0 && !xy) || nprobes > 4096)
        return set_error(IFX_ERR_ARG, "ifx_set_history: bad argument");
    if (!method(S)) return set_error(IFX_ERR_STATE, "ifx_set_history needs a METHOD-mode solver");
    SIO_CUDA(cudaSetDevice(S->device));
    SIO_TRY(finish_pending(S));
    Instance& I = S->inst[inst];
    InstDev& d = I.dev;
    const size_t old_bytes = (size_t)d.hist_cap * d.hist_w * sizeof(double) + (size_t)d.nprobe * sizeof(int);
    free_tracked(S, d.hist);
    free_tracked(S, (void*)d.probe_cell);
    S->device_bytes -= std::min(S->device_bytes, old_bytes);
    d.hist = nullptr;
    d.probe_cell = nullptr;
    d.hist_cap = d.hist_w = d.nprobe = 0;
    if (capacity > 0) {
        const int w = 3 + 3 * nprobes;
        void* h = nullptr;
        SIO_TRY(alloc_tracked(S, &h, (size_t)capacity * w * sizeof(double)));
        SIO_CUDA(cudaMemsetAsync(h, 0, (size_t)capacity * w * sizeof(double), S->stream));
        d.hist = (double*)h;
        if (nprobes > 0) {
            std::vector<int> pc(nprobes);
            for (int k = 0; k < nprobes; k++)
                pc[k] = nearest(I.xc, xy[2 * k]) + nearest(I.yc, xy[2 * k + 1]) * I.pitch;
            void* c = nullptr;
            SIO_TRY(alloc_tracked(S, &c, (size_t)nprobes * sizeof(int)));
            SIO_CUDA(cudaMemcpyAsync(c, pc.data(), pc.size() * sizeof(int), cudaMemcpyHostToDevice, S->stream));
            SIO_CUDA(cudaStreamSynchronize(S->stream));
            d.probe_cell = (const int*)c;
        }
        d.hist_cap = capacity;
        d.hist_w = w;
        d.nprobe = nprobes;
    }
    SIO_CUDA(cudaMemcpyAsync(S->dI + inst, &d, sizeof(InstDev), cudaMemcpyHostToDevice, S->stream));
    // the record count restarts with the new buffer
    InstState st;
    SIO_CUDA(cudaMemcpyAsync(&st, S->dS + inst, sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
    SIO_CUDA(cudaStreamSynchronize(S->stream));
    st.hist_n = 0;
    SIO_CUDA(cudaMemcpyAsync(S->dS + inst, &st, sizeof(InstState), cudaMemcpyHostToDevice, S->stream));
    SIO_CUDA(cudaStreamSynchronize(S->stream));
    return IFX_OK;
}

extern "C" ifx_status ifx_get_probe_cells(ifx_solver* S, int inst, int cap, int* i, int* j, int* n) {
    SIO_TRY(check_inst(S, inst, "ifx_get_probe_cells"));
    if (!n || (cap > 0 && (!i || !j))) return set_error(IFX_ERR_ARG, "ifx_get_probe_cells: bad argument");
    const Instance& I = S->inst[inst];
    const InstDev& d = I.dev;
    *n = d.nprobe;
    if (d.nprobe == 0 || cap <= 0) return IFX_OK;
    std::vector<int> pc(d.nprobe);
    SIO_CUDA(cudaSetDevice(S->device));
    SIO_CUDA(cudaMemcpy(pc.data(), d.probe_cell, pc.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int k = 0; k < d.nprobe && k < cap; k++) {
        i[k] = pc[k] % I.pitch;
        j[k] = pc[k] / I.pitch;
    }
    return IFX_OK;
}

extern "C" ifx_status ifx_get_history(ifx_solver* S, int inst, int cap, double* rows, int* n, int* width) {
    SIO_TRY(check_inst(S, inst, "ifx_get_history"));
    if (!n || (cap > 0 && !rows)) return set_error(IFX_ERR_ARG, "ifx_get_history: bad argument");
    SIO_CUDA(cudaSetDevice(S->device));
    SIO_TRY(finish_pending(S));
    const InstDev& d = S->inst[inst].dev;
    if (width) *width = d.hist_w;
    *n = 0;
    if (d.hist_cap == 0) return IFX_OK;
    InstState st;
    SIO_CUDA(cudaMemcpyAsync(&st, S->dS + inst, sizeof(InstState), cudaMemcpyDeviceToHost, S->stream));
    SIO_CUDA(cudaStreamSynchronize(S->stream));
    const long long have = std::min<long long>(st.hist_n, d.hist_cap);
    const long long take = std::min<long long>(have, std::max(cap, 0));
    // the newest `take` records, oldest first
    std::vector<double> all((size_t)d.hist_cap * d.hist_w);
    SIO_CUDA(cudaMemcpy(all.data(), d.hist, all.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (long long r = 0; r < take; r++) {
        const long long rec = st.hist_n - take + r;
        const size_t slot = (size_t)(rec % d.hist_cap);
        std::memcpy(rows + (size_t)r * d.hist_w, all.data() + slot * d.hist_w, d.hist_w * sizeof(double));
    }
    *n = (int)take;
    return IFX_OK;
}

namespace {
ifx_status history_rows(ifx_solver* S, int inst, std::vector<double>& rows, int& n, int& w) {
    const InstDev& d = S->inst[inst].dev;
    rows.assign((size_t)std::max(1, d.hist_cap) * std::max(1, d.hist_w), 0.0);
    return ifx_get_history(S, inst, d.hist_cap, rows.data(), &n, &w);
}
}  // namespace

extern "C" ifx_status ifx_write_probe_file(ifx_solver* S, int inst, const char* path) {
    SIO_TRY(check_inst(S, inst, "ifx_write_probe_file"));
    if (!path) return set_error(IFX_ERR_ARG, "ifx_write_probe_file: bad argument");
    std::vector<double> rows;
    int n = 0, w = 0;
    SIO_TRY(history_rows(S, inst, rows, n, w));
    const Instance& I = S->inst[inst];
    const int np = I.dev.nprobe;
    std::vector<int> pi(std::max(np, 1)), pj(std::max(np, 1));
    int got = 0;
    SIO_TRY(ifx_get_probe_cells(S, inst, np, pi.data(), pj.data(), &got));
    FILE* f = std::fopen(path, "w");
    if (!f) return set_error(IFX_ERR_IO, std::string("ifx_write_probe_file: cannot write ") + path);
    // header: count, locations (all x, then all y: the cell centres used),
    // then the cell indices i and j (0-based, ghost cell = 0)
    std::fprintf(f, " %d", np);
    for (int k = 0; k < np; k++) std::fprintf(f, " %.10g", I.xc[pi[k]]);
    for (int k = 0; k < np; k++) std::fprintf(f, " %.10g", I.yc[pj[k]]);
    for (int k = 0; k < np; k++) std::fprintf(f, " %d", pi[k]);
    for (int k = 0; k < np; k++) std::fprintf(f, " %d", pj[k]);
    std::fprintf(f, "\n\n Time  U   V  P\n");
    for (int r = 0; r < n; r++) {
        const double* rec = rows.data() + (size_t)r * w;
        std::fprintf(f, "%.10g", rec[0] * I.cfg.dt);
        for (int k = 0; k < np; k++) std::fprintf(f, " %.17g %.17g %.17g", rec[3 + 3 * k], rec[4 + 3 * k], rec[5 + 3 * k]);
        std::fprintf(f, "\n");
    }
    if (std::fclose(f) != 0) return set_error(IFX_ERR_IO, std::string("ifx_write_probe_file: cannot write ") + path);
    return IFX_OK;
}

extern "C" ifx_status ifx_write_force_file(ifx_solver* S, int inst, const char* path) {
    SIO_TRY(check_inst(S, inst, "ifx_write_force_file"));
    if (!path) return set_error(IFX_ERR_ARG, "ifx_write_force_file: bad argument");
    std::vector<double> rows;
    int n = 0, w = 0;
    SIO_TRY(history_rows(S, inst, rows, n, w));
    FILE* f = std::fopen(path, "w");
    if (!f) return set_error(IFX_ERR_IO, std::string("ifx_write_force_file: cannot write ") + path);
    std::fprintf(f, " Time  Cd  Cl\n");
    for (int r = 0; r < n; r++) {
        const double* rec = rows.data() + (size_t)r * w;
        std::fprintf(f, "%.10g %.17g %.17g\n", rec[0] * S->inst[inst].cfg.dt, rec[1], rec[2]);
    }
    if (std::fclose(f) != 0) return set_error(IFX_ERR_IO, std::string("ifx_write_force_file: cannot write ") + path);
    return IFX_OK;
}
