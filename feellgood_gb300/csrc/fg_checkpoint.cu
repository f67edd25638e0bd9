// Full-precision checkpoint and resume of a context (no counterpart in the reference, whose
// .sol snapshots keep u and phi to the output precision and drop v and phiv).
//
// File layout (little-endian, fields written one by one, no padding):
//   "FGGPUCK1" | u32 version | i32 n_nodes, n_mag_tets, precision, solver_lpr,
//   solver_blocks, fmm_depth, solver_threads (version 2; version 1 ends at fmm_depth) |
//   meta: f64 t0, t, dt, dt_soft_max | i64 steps,
//   output_index | u32 rng_seed | i64 rng_draws | f64 E[4] | f64 u[3n], v[3n], phi[n],
//   phiv[n] (CURRENT, node order of the set-up mesh) | u64 FNV-1a of all preceding bytes
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fg_internal.h"

namespace fg {
int fmm_info(const Ctx &c, int *L, int *nleaf, double *n_m2l, double *n_p2p);
}

namespace {

constexpr char MAGIC[8] = {'F', 'G', 'G', 'P', 'U', 'C', 'K', '1'};
constexpr uint32_t VERSION = 2;  // 2: solver_threads after fmm_depth (1 is still read)

struct Writer {
    std::vector<unsigned char> buf;
    template <typename T> void put(const T &v) {
        const unsigned char *p = reinterpret_cast<const unsigned char *>(&v);
        buf.insert(buf.end(), p, p + sizeof(T));
    }
    void put_bytes(const void *p, size_t n) {
        const unsigned char *q = static_cast<const unsigned char *>(p);
        buf.insert(buf.end(), q, q + n);
    }
};

struct Reader {
    const std::vector<unsigned char> &buf;
    size_t pos = 0;
    bool ok = true;
    explicit Reader(const std::vector<unsigned char> &b) : buf(b) {}
    template <typename T> T get() {
        T v{};
        if (pos + sizeof(T) > buf.size()) { ok = false; return v; }
        std::memcpy(&v, buf.data() + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    void get_bytes(void *p, size_t n) {
        if (pos + n > buf.size()) { ok = false; return; }
        std::memcpy(p, buf.data() + pos, n);
        pos += n;
    }
};

uint64_t fnv1a(const unsigned char *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t k = 0; k < n; k++) {
        h ^= p[k];
        h *= 1099511628211ull;
    }
    return h;
}

void put_header(Writer &w, const fg_checkpoint_shape &s, const fg_checkpoint_meta &m) {
    w.put_bytes(MAGIC, 8);
    w.put(VERSION);
    w.put<int32_t>(s.n_nodes); w.put<int32_t>(s.n_mag_tets); w.put<int32_t>(s.precision);
    w.put<int32_t>(s.solver_lpr); w.put<int32_t>(s.solver_blocks); w.put<int32_t>(s.fmm_depth);
    w.put<int32_t>(s.solver_threads);
    w.put(m.t0); w.put(m.t); w.put(m.dt); w.put(m.dt_soft_max);
    w.put<int64_t>(m.steps); w.put<int64_t>(m.output_index);
    w.put<uint32_t>(m.rng_seed); w.put<int64_t>(m.rng_draws);
    for (double e : m.E) w.put(e);
}

// Reads and checks magic, version and checksum; leaves the reader after the header.
int get_header(const std::string &path, std::vector<unsigned char> &buf, Reader &r, fg_checkpoint_shape &s,
               fg_checkpoint_meta &m) {
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return FG_EIO;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 16) { std::fclose(f); return FG_EIO; }
    buf.resize((size_t)n);
    const size_t got = std::fread(buf.data(), 1, buf.size(), f);
    std::fclose(f);
    if (got != buf.size()) return FG_EIO;
    uint64_t stored;
    std::memcpy(&stored, buf.data() + buf.size() - 8, 8);
    if (fnv1a(buf.data(), buf.size() - 8) != stored) return FG_EIO;
    char magic[8];
    r.get_bytes(magic, 8);
    if (std::memcmp(magic, MAGIC, 8) != 0) return FG_EIO;
    const uint32_t version = r.get<uint32_t>();
    if (version != 1 && version != VERSION) return FG_EIO;
    s.n_nodes = r.get<int32_t>(); s.n_mag_tets = r.get<int32_t>(); s.precision = r.get<int32_t>();
    s.solver_lpr = r.get<int32_t>(); s.solver_blocks = r.get<int32_t>(); s.fmm_depth = r.get<int32_t>();
    s.solver_threads = version >= 2 ? r.get<int32_t>() : 0;
    m.t0 = r.get<double>(); m.t = r.get<double>(); m.dt = r.get<double>(); m.dt_soft_max = r.get<double>();
    m.steps = r.get<int64_t>(); m.output_index = r.get<int64_t>();
    m.rng_seed = r.get<uint32_t>(); m.rng_draws = r.get<int64_t>();
    for (double &e : m.E) e = r.get<double>();
    return r.ok ? FG_OK : FG_EIO;
}

}  // namespace

extern "C" {

int fg_checkpoint_save(fg_ctx *h, const char *path, const fg_checkpoint_meta *meta) {
    if (!h || !path || !meta) return FG_EINVAL;
    fg::Ctx &c = h->c;
    if (c.batch) {
        c.err = "fg_checkpoint_save: not available for batch contexts";
        return FG_EINVAL;
    }
    fg_checkpoint_shape s{};
    s.n_nodes = c.nn;
    s.n_mag_tets = c.nmt;
    s.precision = c.opts.precision;
    if (c.opts.precision == FG_PREC_FP32_REFINE) {
        s.solver_lpr = c.lpr;
        s.solver_blocks = c.mixed_grid;
        s.solver_threads = c.mixed_threads;
    }
    if (c.fmm) {
        int L = 0, nl = 0;
        double a = 0, b = 0;
        fg::fmm_info(c, &L, &nl, &a, &b);
        s.fmm_depth = L;
    }
    const size_t n = (size_t)c.nn;
    std::vector<double> u(3 * n), v(3 * n), phi(n), phiv(n);
    int st = fg_get_state(h, 0, u.data(), v.data(), phi.data(), phiv.data());
    if (st != FG_OK) return st;
    Writer w;
    put_header(w, s, *meta);
    w.put_bytes(u.data(), u.size() * sizeof(double));
    w.put_bytes(v.data(), v.size() * sizeof(double));
    w.put_bytes(phi.data(), phi.size() * sizeof(double));
    w.put_bytes(phiv.data(), phiv.size() * sizeof(double));
    w.put(fnv1a(w.buf.data(), w.buf.size()));
    // write then rename: a reader never sees a half-written checkpoint
    const std::string tmp = std::string(path) + ".tmp";
    std::FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) {
        c.err = "fg_checkpoint_save: cannot open " + tmp;
        return FG_EIO;
    }
    const bool ok = std::fwrite(w.buf.data(), 1, w.buf.size(), f) == w.buf.size();
    if (std::fclose(f) != 0 || !ok || std::rename(tmp.c_str(), path) != 0) {
        c.err = std::string("fg_checkpoint_save: cannot write ") + path;
        return FG_EIO;
    }
    return FG_OK;
}

int fg_checkpoint_peek(const char *path, fg_checkpoint_shape *shape, fg_checkpoint_meta *meta) {
    if (!path) return FG_EINVAL;
    std::vector<unsigned char> buf;
    Reader r(buf);
    fg_checkpoint_shape s{};
    fg_checkpoint_meta m{};
    const int st = get_header(path, buf, r, s, m);
    if (st != FG_OK) return st;
    if (shape) *shape = s;
    if (meta) *meta = m;
    return FG_OK;
}

int fg_checkpoint_load(fg_ctx *h, const char *path, fg_checkpoint_meta *meta) {
    if (!h || !path) return FG_EINVAL;
    fg::Ctx &c = h->c;
    std::vector<unsigned char> buf;
    Reader r(buf);
    fg_checkpoint_shape s{};
    fg_checkpoint_meta m{};
    int st = get_header(path, buf, r, s, m);
    if (st != FG_OK) {
        c.err = std::string("fg_checkpoint_load: unreadable or corrupt checkpoint ") + path;
        return st;
    }
    if (s.n_nodes != c.nn || s.n_mag_tets != c.nmt) {
        c.err = "fg_checkpoint_load: the checkpoint belongs to another mesh";
        return FG_EINVAL;
    }
    const size_t n = (size_t)c.nn;
    std::vector<double> u(3 * n), v(3 * n), phi(n), phiv(n);
    r.get_bytes(u.data(), u.size() * sizeof(double));
    r.get_bytes(v.data(), v.size() * sizeof(double));
    r.get_bytes(phi.data(), phi.size() * sizeof(double));
    r.get_bytes(phiv.data(), phiv.size() * sizeof(double));
    if (!r.ok || r.pos + 8 != buf.size()) {
        c.err = "fg_checkpoint_load: truncated checkpoint";
        return FG_EIO;
    }
    st = fg_set_state(h, u.data(), v.data(), phi.data(), phiv.data());
    if (st != FG_OK) return st;
    if (meta) *meta = m;
    return FG_OK;
}

}  // extern "C"
