// wf_format.cpp -- version-1 MOCCa wavefunction files (include/mocca_wf.h):
// Fortran unformatted sequential records and the record order of
// WriteMOCCa_v1 / ReadMOCCa_v1 (src/InOut.f90:905-1416).  Host code only.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>

#include "wf_format.h"

namespace mg {

namespace {

// gfortran's largest subrecord payload (2^31 - 9 bytes)
constexpr long long kMaxSub = 2147483639LL;
constexpr int kForceLen = 200;   // character(len=200) :: afor (src/Force.f90:23)

void put_i32(unsigned char* p, int32_t v) {
    const uint32_t u = (uint32_t)v;
    p[0] = (unsigned char)(u & 0xff);
    p[1] = (unsigned char)((u >> 8) & 0xff);
    p[2] = (unsigned char)((u >> 16) & 0xff);
    p[3] = (unsigned char)((u >> 24) & 0xff);
}

int32_t get_i32(const unsigned char* p) {
    const uint32_t u = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
                       ((uint32_t)p[3] << 24);
    return (int32_t)u;
}

// Record markers are assembled byte by byte; payload doubles and ints are
// copied as the host stores them, which is little-endian order on both
// hosts this library builds for (x86-64, aarch64).  A big-endian host is
// refused rather than written wrong.
bool host_is_little_endian() {
    const uint32_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

// One logical record assembled in memory, then written as subrecords.
class RecordWriter {
  public:
    explicit RecordWriter(FILE* f) : f_(f) {}
    void i32(int v) {
        unsigned char b[4];
        put_i32(b, v);
        raw(b, 4);
    }
    void logical(int v) { i32(v ? 1 : 0); }
    void f64(double v) { raw(&v, 8); }
    void f64s(const double* p, long long n) { raw(p, (size_t)n * 8); }
    void i32s(const int* p, long long n) {
        for (long long k = 0; k < n; ++k) i32(p[k]);
    }
    void raw(const void* p, size_t n) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        buf_.insert(buf_.end(), c, c + n);
    }
    // write the assembled payload as one record and start the next
    bool end() {
        const long long n = (long long)buf_.size();
        long long pos = 0;
        bool first = true;
        do {
            const long long len = std::min(kMaxSub, n - pos);
            const bool last = pos + len == n;
            unsigned char m[4];
            put_i32(m, (int32_t)(last ? len : -len));
            if (std::fwrite(m, 1, 4, f_) != 4) return false;
            if (len > 0 && std::fwrite(buf_.data() + pos, 1, (size_t)len, f_) != (size_t)len)
                return false;
            put_i32(m, (int32_t)(first ? len : -len));
            if (std::fwrite(m, 1, 4, f_) != 4) return false;
            pos += len;
            first = false;
        } while (pos < n);
        buf_.clear();
        return true;
    }

  private:
    FILE* f_;
    std::vector<unsigned char> buf_;
};

// Sequential reader of logical records; the cursor reads items off the
// current record and fails when the record is too short.
class RecordReader {
  public:
    explicit RecordReader(FILE* f) : f_(f) {}
    // 1: a record was read; 0: end of file before a record; -1: damaged file
    int next() {
        buf_.clear();
        pos_ = 0;
        bool first = true;
        for (;;) {
            unsigned char m[4];
            const size_t got = std::fread(m, 1, 4, f_);
            if (got == 0 && first) return 0;
            if (got != 4) return -1;
            const int32_t lead = get_i32(m);
            const long long len = lead < 0 ? -(long long)lead : (long long)lead;
            const size_t old = buf_.size();
            try {
                buf_.resize(old + (size_t)len);
            } catch (const std::bad_alloc&) {
                return -1;
            }
            if (len > 0 && std::fread(buf_.data() + old, 1, (size_t)len, f_) != (size_t)len)
                return -1;
            if (std::fread(m, 1, 4, f_) != 4) return -1;
            const int32_t trail = get_i32(m);
            const long long tl = trail < 0 ? -(long long)trail : (long long)trail;
            if (tl != len || (trail < 0) == first) return -1;
            first = false;
            if (lead >= 0) return 1;
        }
    }
    size_t size() const { return buf_.size(); }
    bool has(size_t n) const { return pos_ + n <= buf_.size(); }
    int i32() {
        const int v = get_i32(buf_.data() + pos_);
        pos_ += 4;
        return v;
    }
    double f64() {
        double v;
        std::memcpy(&v, buf_.data() + pos_, 8);
        pos_ += 8;
        return v;
    }
    void f64s(double* p, long long n) {
        std::memcpy(p, buf_.data() + pos_, (size_t)n * 8);
        pos_ += (size_t)n * 8;
    }
    void i32s(int* p, long long n) {
        for (long long k = 0; k < n; ++k) p[k] = i32();
    }
    void bytes(char* p, size_t n) {
        std::memcpy(p, buf_.data() + pos_, n);
        pos_ += n;
    }

  private:
    FILE* f_;
    std::vector<unsigned char> buf_;
    size_t pos_ = 0;
};

struct FileCloser {
    void operator()(FILE* f) const {
        if (f) std::fclose(f);
    }
};

long long mesh_v(const mg_wf_header& h) { return (long long)h.nx * h.ny * h.nz; }

// element counts of the time-odd density records, in units of V
constexpr int kOddV[5] = {12, 30, 14, 6, 6};

}  // namespace

bool wf_field_is_int(int field) {
    return field == MG_WF_SPWF_INT || field == MG_WF_BLOCKSIZES || field == MG_WF_COLUMNS ||
           field == MG_WF_MOMENT_INT;
}

void wf_derive_shapes(mg_wf_header& h) {
    h.hfb_size = h.trc ? 2 * h.nwt : h.nwt;   // src/Pairing.f90:400-405
    h.pindex = h.pc ? 2 : 1;                  // PrepareHFBModule, src/HFB.f90:254-255
    h.iindex = h.ic ? 2 : 1;
    if (h.can_blocks <= 0) h.can_blocks = h.pindex * h.iindex;
    h.version = 1;
}

long long wf_field_count(const mg_wf_header& h, int field) {
    const long long V = mesh_v(h), n = h.nwt, m = h.hfb_size;
    switch (field) {
        case MG_WF_GRIDS: return n * 4 * V;
        case MG_WF_SPWF_REAL: return n * 7;
        case MG_WF_SPWF_INT: return n * 5;
        case MG_WF_RHO: case MG_WF_LAPRHO: case MG_WF_TAU: case MG_WF_NABLAJ: return 2 * V;
        case MG_WF_DERRHO: return 6 * V;
        case MG_WF_JMUNU: return h.has_jmunu ? 18 * V : 0;
        case MG_WF_ODD1: case MG_WF_ODD2: case MG_WF_ODD3: case MG_WF_ODD4: case MG_WF_ODD5: {
            const int k = field - MG_WF_ODD1;
            return (h.odd_records >> k) & 1 ? kOddV[k] * V : 0;
        }
        case MG_WF_CUTOFFS: return h.has_cutoffs ? n : 0;
        case MG_WF_BLOCKSIZES: return (long long)h.pindex * h.iindex;
        case MG_WF_U: case MG_WF_V: return 2 * m * 2 * m * 4;
        case MG_WF_COLUMNS: return m * h.pindex * h.iindex;
        case MG_WF_RHOHFB: case MG_WF_KAPPAHFB: return 2 * m * m * 4;
        case MG_WF_CANTRANSFO: return 2 * m * m * h.can_blocks;
        case MG_WF_MOMENT_INT: return (long long)h.n_moments * 5;
        case MG_WF_MOMENT_REAL: return (long long)h.n_moments * 22;
        default: return 0;
    }
}

void wf_allocate(mg_wf& w) {
    for (int f = 0; f < MG_WF_NFIELDS; ++f) {
        const long long c = wf_field_count(w.h, f);
        if (wf_field_is_int(f)) {
            w.i[f].assign((size_t)c, 0);
            w.d[f].clear();
        } else {
            w.d[f].assign((size_t)c, 0.0);
            w.i[f].clear();
        }
    }
}

namespace {

bool valid_shape(const mg_wf_header& h) {
    if (h.nx < 1 || h.ny < 1 || h.nz < 1 || h.nwt < 0) return false;
    // 4V doubles of one spwf grid must fit a record count and memory
    const long long V = mesh_v(h);
    return V <= (1LL << 31) / 32 && h.nwt <= (1 << 20) && h.n_moments >= 0 &&
           h.n_moments <= 1024;
}

int load(const char* path, mg_wf& w) {
    if (!host_is_little_endian()) return MG_ERR_IO;
    std::unique_ptr<FILE, FileCloser> fp(std::fopen(path, "rb"));
    if (!fp) return MG_ERR_IO;
    RecordReader r(fp.get());
    mg_wf_header& h = w.h;
    h = mg_wf_header{};
    auto rec = [&](size_t need) { return r.next() == 1 && r.has(need); };
    // 1-5: version, convergence, mesh, symmetries, particle numbers
    if (!rec(4)) return MG_ERR_IO;
    if (r.i32() != 1) return MG_ERR_IO;   // File format has unrecognised version
    if (!rec(16)) return MG_ERR_IO;
    h.energy = r.f64();
    h.denergy = r.f64();
    if (!rec(20)) return MG_ERR_IO;
    h.nx = r.i32();
    h.ny = r.i32();
    h.nz = r.i32();
    h.dx = r.f64();
    if (!rec(20)) return MG_ERR_IO;
    h.trc = r.i32() != 0;
    h.pc = r.i32() != 0;
    h.sc = r.i32() != 0;
    h.tsc = r.i32() != 0;
    h.ic = r.i32() != 0;
    if (!rec(20)) return MG_ERR_IO;
    h.nwt = r.i32();
    h.neutrons = r.f64();
    h.protons = r.f64();
    if (!valid_shape(h)) return MG_ERR_IO;
    wf_derive_shapes(h);
    const long long V = mesh_v(h);
    // the optional records are sized once read; start with none of them
    h.has_jmunu = 0;
    h.odd_records = 0;
    h.has_cutoffs = 0;
    h.n_moments = 0;
    wf_allocate(w);
    // spwfs (ReadSpwf, src/Spwf.f90:2263-2287)
    for (int k = 0; k < h.nwt; ++k) {
        if (!rec((size_t)(4 * V * 8))) return MG_ERR_IO;
        r.f64s(w.d[MG_WF_GRIDS].data() + (size_t)k * 4 * V, 4 * V);
        if (!rec(7 * 8 + 5 * 4)) return MG_ERR_IO;
        r.f64s(w.d[MG_WF_SPWF_REAL].data() + (size_t)k * 7, 7);
        r.i32s(w.i[MG_WF_SPWF_INT].data() + (size_t)k * 5, 5);
        const int iso = w.i[MG_WF_SPWF_INT][(size_t)k * 5];
        if (iso != 1 && iso != -1) return MG_ERR_IO;   // Wrong isospin on file
    }
    // densities (ReadDensity, src/Densities.f90:1242-1348): the optional
    // records read as absent when empty or too short, as its iostat
    // handling zeroes them
    if (!rec((size_t)(10 * V * 8))) return MG_ERR_IO;
    r.f64s(w.d[MG_WF_RHO].data(), 2 * V);
    r.f64s(w.d[MG_WF_DERRHO].data(), 6 * V);
    r.f64s(w.d[MG_WF_LAPRHO].data(), 2 * V);
    if (!rec((size_t)(2 * V * 8))) return MG_ERR_IO;
    r.f64s(w.d[MG_WF_TAU].data(), 2 * V);
    if (!rec((size_t)(2 * V * 8))) return MG_ERR_IO;
    r.f64s(w.d[MG_WF_NABLAJ].data(), 2 * V);
    if (r.next() != 1) return MG_ERR_IO;
    if (r.has((size_t)(18 * V * 8))) {
        h.has_jmunu = 1;
        w.d[MG_WF_JMUNU].resize((size_t)(18 * V));
        r.f64s(w.d[MG_WF_JMUNU].data(), 18 * V);
    }
    for (int k = 0; k < 5; ++k) {
        if (r.next() != 1) return MG_ERR_IO;
        if (r.has((size_t)(kOddV[k] * V * 8))) {
            h.odd_records |= 1 << k;
            w.d[MG_WF_ODD1 + k].resize((size_t)(kOddV[k] * V));
            r.f64s(w.d[MG_WF_ODD1 + k].data(), kOddV[k] * V);
        }
    }
    // 6: finite-difference orders; 7-10: the force
    if (!rec(12)) return MG_ERR_IO;
    h.fd_order = r.i32();
    h.fd_lap_order = r.i32();
    h.coulomb_lap_order = r.i32();
    if (!rec(kForceLen)) return MG_ERR_IO;
    {
        char name[kForceLen + 1];
        r.bytes(name, kForceLen);
        int n = kForceLen;
        while (n > 0 && (name[n - 1] == ' ' || name[n - 1] == '\0')) --n;
        name[n] = '\0';
        std::memcpy(h.force, name, (size_t)n + 1);
    }
    if (!rec(14 * 8)) return MG_ERR_IO;
    for (double& x : h.skyrme) x = r.f64();
    if (!rec(kForceLen + 3 * 8 + 2 * 4)) return MG_ERR_IO;
    {
        char skip[kForceLen];
        r.bytes(skip, kForceLen);
    }
    h.hbar = r.f64();
    h.hbm[0] = r.f64();
    h.hbm[1] = r.f64();
    h.com1body = r.i32();
    h.com2body = r.i32();
    if (!rec(28 * 8)) return MG_ERR_IO;
    for (double& x : h.coef) x = r.f64();
    // 11-13: pairing
    if (!rec(4 + 6 * 8)) return MG_ERR_IO;
    h.pairing_type = r.i32();
    for (double& x : h.pairing_strength) x = r.f64();
    for (double& x : h.pairing_alpha) x = r.f64();
    for (double& x : h.pairing_cut) x = r.f64();
    if (r.next() != 1) return MG_ERR_IO;
    if (h.nwt > 0 && r.has((size_t)h.nwt * 8)) {
        h.has_cutoffs = 1;
        w.d[MG_WF_CUTOFFS].resize((size_t)h.nwt);
        r.f64s(w.d[MG_WF_CUTOFFS].data(), h.nwt);
    }
    if (!rec(4 * 8)) return MG_ERR_IO;
    h.fermi[0] = r.f64();
    h.fermi[1] = r.f64();
    h.ln_lambda[0] = r.f64();
    h.ln_lambda[1] = r.f64();
    // 14-18: HFB matrices (read as ReadMOCCa_v1's PairingType 2 branch)
    auto read_field = [&](int f) {
        const long long c = wf_field_count(h, f);
        if (wf_field_is_int(f))
            r.i32s(w.i[f].data(), c);
        else
            r.f64s(w.d[f].data(), c);
        return c;
    };
    auto bytes_of = [&](int f) {
        return (size_t)wf_field_count(h, f) * (wf_field_is_int(f) ? 4 : 8);
    };
    if (!rec(bytes_of(MG_WF_BLOCKSIZES))) return MG_ERR_IO;
    read_field(MG_WF_BLOCKSIZES);
    if (!rec(bytes_of(MG_WF_U) + bytes_of(MG_WF_V))) return MG_ERR_IO;
    read_field(MG_WF_U);
    read_field(MG_WF_V);
    if (!rec(bytes_of(MG_WF_COLUMNS))) return MG_ERR_IO;
    read_field(MG_WF_COLUMNS);
    if (!rec(bytes_of(MG_WF_RHOHFB) + bytes_of(MG_WF_KAPPAHFB))) return MG_ERR_IO;
    read_field(MG_WF_RHOHFB);
    read_field(MG_WF_KAPPAHFB);
    if (!rec(bytes_of(MG_WF_CANTRANSFO))) return MG_ERR_IO;
    {
        // GuessHFBMatrices allocates CanTransfo with 2 x 2 blocks whatever the
        // symmetries: keep the whole blocks the record holds (at most 4)
        const size_t blk = (size_t)h.hfb_size * h.hfb_size * 16;
        const int have = blk ? (int)std::min<size_t>(4, r.size() / blk) : h.can_blocks;
        h.can_blocks = std::max(h.can_blocks, have);
        w.d[MG_WF_CANTRANSFO].resize((size_t)wf_field_count(h, MG_WF_CANTRANSFO));
        read_field(MG_WF_CANTRANSFO);
    }
    // 19: cranking
    if (!rec(6 * 8)) return MG_ERR_IO;
    for (double& x : h.omega) x = r.f64();
    for (double& x : h.crank_values) x = r.f64();
    // moments up to the end of the file (ReadMoment, src/Moments.f90:3365-3427)
    for (;;) {
        const int st = r.next();
        if (st == 0) break;
        if (st < 0 || !r.has(20)) return MG_ERR_IO;
        int mi[5];
        r.i32s(mi, 5);
        if (!rec(22 * 8)) return MG_ERR_IO;
        double mr[22];
        r.f64s(mr, 22);
        w.i[MG_WF_MOMENT_INT].insert(w.i[MG_WF_MOMENT_INT].end(), mi, mi + 5);
        w.d[MG_WF_MOMENT_REAL].insert(w.d[MG_WF_MOMENT_REAL].end(), mr, mr + 22);
        ++h.n_moments;
    }
    return MG_OK;
}

int save(const mg_wf& w, const char* path) {
    if (!host_is_little_endian()) return MG_ERR_IO;
    const mg_wf_header& h = w.h;
    for (int f = 0; f < MG_WF_NFIELDS; ++f) {
        const size_t have = wf_field_is_int(f) ? w.i[f].size() : w.d[f].size();
        if ((long long)have != wf_field_count(h, f)) return MG_ERR_STATE;
    }
    std::unique_ptr<FILE, FileCloser> fp(std::fopen(path, "wb"));
    if (!fp) return MG_ERR_IO;
    RecordWriter o(fp.get());
    bool ok = true;
    auto end = [&]() { ok = ok && o.end(); };
    const long long V = mesh_v(h);
    o.i32(1);
    end();
    o.f64(h.energy);
    o.f64(h.denergy);
    end();
    o.i32(h.nx);
    o.i32(h.ny);
    o.i32(h.nz);
    o.f64(h.dx);
    end();
    o.logical(h.trc);
    o.logical(h.pc);
    o.logical(h.sc);
    o.logical(h.tsc);
    o.logical(h.ic);
    end();
    o.i32(h.nwt);
    o.f64(h.neutrons);
    o.f64(h.protons);
    end();
    for (int k = 0; k < h.nwt; ++k) {
        o.f64s(w.d[MG_WF_GRIDS].data() + (size_t)k * 4 * V, 4 * V);
        end();
        o.f64s(w.d[MG_WF_SPWF_REAL].data() + (size_t)k * 7, 7);
        o.i32s(w.i[MG_WF_SPWF_INT].data() + (size_t)k * 5, 5);
        end();
    }
    auto field = [&](int f) {
        if (wf_field_is_int(f))
            o.i32s(w.i[f].data(), (long long)w.i[f].size());
        else
            o.f64s(w.d[f].data(), (long long)w.d[f].size());
    };
    field(MG_WF_RHO);
    field(MG_WF_DERRHO);
    field(MG_WF_LAPRHO);
    end();
    field(MG_WF_TAU);
    end();
    field(MG_WF_NABLAJ);
    end();
    field(MG_WF_JMUNU);   // empty when absent
    end();
    for (int k = 0; k < 5; ++k) {
        field(MG_WF_ODD1 + k);
        end();
    }
    o.i32(h.fd_order);
    o.i32(h.fd_lap_order);
    o.i32(h.coulomb_lap_order);
    end();
    char name[kForceLen];
    std::memset(name, ' ', kForceLen);
    std::memcpy(name, h.force, std::min<size_t>(kForceLen, strnlen(h.force, sizeof(h.force))));
    o.raw(name, kForceLen);
    end();
    for (double x : h.skyrme) o.f64(x);
    end();
    o.raw(name, kForceLen);
    o.f64(h.hbar);
    o.f64(h.hbm[0]);
    o.f64(h.hbm[1]);
    o.i32(h.com1body);
    o.i32(h.com2body);
    end();
    for (double x : h.coef) o.f64(x);
    end();
    o.i32(h.pairing_type);
    for (double x : h.pairing_strength) o.f64(x);
    for (double x : h.pairing_alpha) o.f64(x);
    for (double x : h.pairing_cut) o.f64(x);
    end();
    field(MG_WF_CUTOFFS);
    end();
    o.f64(h.fermi[0]);
    o.f64(h.fermi[1]);
    o.f64(h.ln_lambda[0]);
    o.f64(h.ln_lambda[1]);
    end();
    field(MG_WF_BLOCKSIZES);
    end();
    field(MG_WF_U);
    field(MG_WF_V);
    end();
    field(MG_WF_COLUMNS);
    end();
    field(MG_WF_RHOHFB);
    field(MG_WF_KAPPAHFB);
    end();
    field(MG_WF_CANTRANSFO);
    end();
    for (double x : h.omega) o.f64(x);
    for (double x : h.crank_values) o.f64(x);
    end();
    for (int k = 0; k < h.n_moments; ++k) {
        o.i32s(w.i[MG_WF_MOMENT_INT].data() + (size_t)k * 5, 4);
        o.logical(w.i[MG_WF_MOMENT_INT][(size_t)k * 5 + 4]);
        end();
        o.f64s(w.d[MG_WF_MOMENT_REAL].data() + (size_t)k * 22, 22);
        end();
    }
    if (!ok) return MG_ERR_IO;
    FILE* f = fp.release();
    return std::fclose(f) == 0 ? MG_OK : MG_ERR_IO;
}

}  // namespace

}  // namespace mg

using namespace mg;

extern "C" int mg_wf_load(const char* path, mg_wf** out) {
    if (!path || !out) return MG_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<mg_wf> w;
    try {
        w.reset(new mg_wf());
        const int st = load(path, *w);
        if (st != MG_OK) return st;
    } catch (const std::bad_alloc&) {
        return MG_ERR_IO;
    }
    *out = w.release();
    return MG_OK;
}

extern "C" int mg_wf_new(const mg_wf_header* h, mg_wf** out) {
    if (!h || !out) return MG_ERR_ARG;
    *out = nullptr;
    mg_wf_header hh = *h;
    if (!valid_shape(hh) || hh.can_blocks < 0 || hh.can_blocks > 4) return MG_ERR_ARG;
    hh.trc = hh.trc != 0;
    hh.pc = hh.pc != 0;
    hh.sc = hh.sc != 0;
    hh.tsc = hh.tsc != 0;
    hh.ic = hh.ic != 0;
    hh.has_jmunu = hh.has_jmunu != 0;
    hh.has_cutoffs = hh.has_cutoffs != 0;
    hh.odd_records &= 31;
    hh.force[sizeof(hh.force) - 1] = '\0';
    wf_derive_shapes(hh);
    try {
        std::unique_ptr<mg_wf> w(new mg_wf());
        w->h = hh;
        wf_allocate(*w);
        *out = w.release();
    } catch (const std::bad_alloc&) {
        return MG_ERR_ARG;
    }
    return MG_OK;
}

extern "C" int mg_wf_save(const mg_wf* wf, const char* path) {
    if (!wf || !path) return MG_ERR_ARG;
    try {
        return save(*wf, path);
    } catch (const std::bad_alloc&) {
        return MG_ERR_IO;
    }
}

extern "C" int mg_wf_free(mg_wf* wf) {
    if (!wf) return MG_ERR_ARG;
    delete wf;
    return MG_OK;
}

extern "C" int mg_wf_get_header(const mg_wf* wf, mg_wf_header* out) {
    if (!wf || !out) return MG_ERR_ARG;
    *out = wf->h;
    return MG_OK;
}

extern "C" int mg_wf_set_scalars(mg_wf* wf, const mg_wf_header* s) {
    if (!wf || !s) return MG_ERR_ARG;
    mg_wf_header& h = wf->h;
    h.energy = s->energy;
    h.denergy = s->denergy;
    h.dx = s->dx;
    h.neutrons = s->neutrons;
    h.protons = s->protons;
    h.fd_order = s->fd_order;
    h.fd_lap_order = s->fd_lap_order;
    h.coulomb_lap_order = s->coulomb_lap_order;
    std::memcpy(h.force, s->force, sizeof(h.force));
    h.force[sizeof(h.force) - 1] = '\0';
    std::copy(s->skyrme, s->skyrme + 14, h.skyrme);
    h.hbar = s->hbar;
    h.hbm[0] = s->hbm[0];
    h.hbm[1] = s->hbm[1];
    h.com1body = s->com1body;
    h.com2body = s->com2body;
    std::copy(s->coef, s->coef + 28, h.coef);
    h.pairing_type = s->pairing_type;
    for (int k = 0; k < 2; ++k) {
        h.pairing_strength[k] = s->pairing_strength[k];
        h.pairing_alpha[k] = s->pairing_alpha[k];
        h.pairing_cut[k] = s->pairing_cut[k];
        h.fermi[k] = s->fermi[k];
        h.ln_lambda[k] = s->ln_lambda[k];
    }
    std::copy(s->omega, s->omega + 3, h.omega);
    std::copy(s->crank_values, s->crank_values + 3, h.crank_values);
    return MG_OK;
}

extern "C" int mg_wf_field(mg_wf* wf, int field, void** data, long long* count) {
    if (!wf || !data || !count || field < 0 || field >= MG_WF_NFIELDS) return MG_ERR_ARG;
    if (wf_field_is_int(field)) {
        *data = wf->i[field].empty() ? nullptr : wf->i[field].data();
        *count = (long long)wf->i[field].size();
    } else {
        *data = wf->d[field].empty() ? nullptr : wf->d[field].data();
        *count = (long long)wf->d[field].size();
    }
    return MG_OK;
}
