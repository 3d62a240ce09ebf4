// uvfits.cu -- visibilities from a FITS random-groups file (the FTS branch of VISGET,
// vis/visget.f:60-68) straight into the SoA arrays the plans take: the header is parsed on the
// host (the checks of fts/ftsgrpre.f and vis/visstd.f, with their messages), the group records
// are read into two pinned host buffers in turn and copied to the device, and one kernel per
// chunk decodes the big-endian words (fts/fti.c fticr_), applies the parameter and array
// scalings (fts/ftsgrpre.f:229-243), takes u, v, w to wavelengths (vis/visstd.f:135-202),
// converts the correlations to Stokes (vis/visconvs.f, visconv2.f, visconvp.f) and keeps one
// Stokes parameter's VIS and WT (vis/visstd.f:260-314).  The file is read while the previous
// chunk is copied and decoded, each chunk by a pool of reader threads (pread of disjoint
// slices), so the read is not bound by one thread's copy out of the page cache.
#include <errno.h>
#include <fcntl.h>
#include <stdio.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

struct sde_uvfits {
    std::string path;
    int64_t data_off = 0;  // byte offset of the first group
    sde_uvfits_desc d{};
    int lgrp = 0, ws = 0, nreg = 0;
    int par_u = -1, par_v = -1, par_w = -1, par_wt = -1;
    std::vector<double> pscal, pzero;
    double bscale = 1.0, bzero = 0.0;
};

namespace {

// ---------------------------------------------------------------------------------------
// Chunk reader: a chunk's bytes are split into one slice per thread and read with pread on
// one descriptor (the calling thread reads slice 0).  The result is the length of the chunk's
// contiguous prefix that was read: a short slice is the end of the file, and what follows it
// is not counted, as a sequential read would stop there.
class ChunkReader {
  public:
    ChunkReader(int fd, int nthreads) : fd_(fd), n_(nthreads), got_((size_t)nthreads, 0) {
        try {
            for (int t = 1; t < n_; t++) th_.emplace_back([this, t] { worker(t); });
        } catch (...) {
            finish();  // the threads that did start are joined before the error propagates
            throw;
        }
    }
    ~ChunkReader() { finish(); }
    // len bytes at file offset off into dst; the contiguous bytes read, or -1 on a read error
    int64_t read(uint8_t *dst, int64_t off, int64_t len) {
        {
            std::lock_guard<std::mutex> l(m_);
            dst_ = dst;
            off_ = off;
            len_ = len;
            pending_ = n_ - 1;
            err_ = false;
            gen_++;
        }
        cv_.notify_all();
        slice(0);
        {
            std::unique_lock<std::mutex> l(m_);
            done_.wait(l, [this] { return pending_ == 0; });
        }
        if (err_) return -1;
        int64_t total = 0;
        for (int t = 0; t < n_; t++) {
            total += got_[(size_t)t];
            if (got_[(size_t)t] < bound(t + 1) - bound(t)) break;
        }
        return total;
    }

  private:
    void finish() {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
            gen_++;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
        th_.clear();
    }
    int64_t bound(int t) const { return len_ * t / n_; }
    void slice(int t) {
        const int64_t a = bound(t), b = bound(t + 1);
        int64_t done = 0;
        while (a + done < b) {
            const ssize_t r = pread(fd_, dst_ + a + done, (size_t)(b - a - done), (off_t)(off_ + a + done));
            if (r < 0 && errno == EINTR) continue;
            if (r < 0) err_ = true;
            if (r <= 0) break;
            done += r;
        }
        got_[(size_t)t] = done;
    }
    void worker(int t) {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
            }
            slice(t);
            std::lock_guard<std::mutex> l(m_);
            if (--pending_ == 0) done_.notify_one();
        }
    }
    const int fd_, n_;
    std::vector<int64_t> got_;
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    uint64_t gen_ = 0;
    bool stop_ = false;
    int pending_ = 0;
    std::atomic<bool> err_{false};
    uint8_t *dst_ = nullptr;
    int64_t off_ = 0, len_ = 0;
};

int reader_threads() {
    const unsigned hw = std::thread::hardware_concurrency();
    return (int)std::min(8u, std::max(1u, hw));
}

// ---------------------------------------------------------------------------------------
// Header.  80-character cards in 2880-byte blocks up to END; "KEYWORD = value / comment".
struct Card {
    bool is_str = false;
    std::string s;  // string value (quotes removed, trailing blanks trimmed) or raw token
    double num = 0.0;
    bool has_num = false;
};

std::string trim(const std::string &x) {
    size_t a = 0, b = x.size();
    while (a < b && x[a] == ' ') a++;
    while (b > a && x[b - 1] == ' ') b--;
    return x.substr(a, b - a);
}

Card parse_value(const char *v, int len) {
    Card c;
    int i = 0;
    while (i < len && v[i] == ' ') i++;
    if (i < len && v[i] == '\'') {
        std::string s;
        for (i++; i < len; i++) {
            if (v[i] == '\'') {
                if (i + 1 < len && v[i + 1] == '\'') {
                    s += '\'';
                    i++;
                } else {
                    break;
                }
            } else {
                s += v[i];
            }
        }
        // trailing blanks are not significant in FITS strings
        while (!s.empty() && s.back() == ' ') s.pop_back();
        c.is_str = true;
        c.s = s;
        return c;
    }
    std::string tok;
    for (; i < len && v[i] != '/'; i++) tok += v[i];
    tok = trim(tok);
    c.s = tok;
    std::string t = tok;
    for (char &ch : t)
        if (ch == 'D' || ch == 'd') ch = 'E';  // Fortran double exponents
    if (!t.empty() && t != "T" && t != "F") {
        char *end = nullptr;
        const double x = strtod(t.c_str(), &end);
        if (end && *end == '\0') {
            c.num = x;
            c.has_num = true;
        }
    }
    return c;
}

struct Header {
    std::map<std::string, Card> cards;
    const Card *get(const std::string &k) const {
        auto it = cards.find(k);
        return it == cards.end() ? nullptr : &it->second;
    }
    bool num(const std::string &k, double *x) const {
        const Card *c = get(k);
        if (!c || !c->has_num) return false;
        *x = c->num;
        return true;
    }
    double num_or(const std::string &k, double dflt) const {
        double x;
        return num(k, &x) ? x : dflt;
    }
    std::string str(const std::string &k) const {
        const Card *c = get(k);
        return c ? c->s : std::string();
    }
    bool logical(const std::string &k) const {
        const Card *c = get(k);
        return c && !c->is_str && c->s == "T";
    }
};

// reads cards up to END; returns the byte offset of the data (next 2880 boundary)
int read_header(FILE *fp, Header *h, int64_t *data_off) {
    char card[81];
    card[80] = '\0';
    int64_t pos = 0;
    for (;;) {
        if (fread(card, 1, 80, fp) != 80) {
            sde_set_error("sde_uvfits_open: no END card (not a FITS file?)");
            return SDE_EINVAL;
        }
        pos += 80;
        std::string key = trim(std::string(card, 8));
        if (key == "END") break;
        if (card[8] == '=' && card[9] == ' ' && !key.empty() && !h->cards.count(key))
            h->cards[key] = parse_value(card + 10, 70);
        if (pos > (int64_t)1 << 24) {
            sde_set_error("sde_uvfits_open: header longer than 16 MB");
            return SDE_EINVAL;
        }
    }
    *data_off = (pos + 2879) / 2880 * 2880;
    return SDE_OK;
}

// ---------------------------------------------------------------------------------------
// Decoding.
enum { CONV_NONE = 0, CONV_AIPS4 = 1, CONV_AIPS2 = 2, CONV_PIPE4 = 3 };

struct UvDecode {
    int lgrp, ws, bitpix, npar, inc, conv, pos;  // pos: position of the wanted Stokes, 0..3
    int par[4];                                  // u, v, w, weight (-1: none)
    double ps[4], pz[4];
    int pid[4];                                  // parameter scaling is the identity
    double bscale, bzero;
    int aid;                                     // array scaling is the identity
    float freq;                                  // SNGL(FREQ)
    int scale_uvw;
};

// word k of a group as fticr_ sees it (fts/fti.c:69-168): big-endian 16/32-bit integer or IEEE
__device__ __forceinline__ double word_raw(const uint8_t *g, int k, int ws, int bitpix, float *fval) {
    if (ws == 2) {
        const uint16_t x = reinterpret_cast<const uint16_t *>(g)[k];
        const uint16_t y = (uint16_t)((x >> 8) | (x << 8));
        return (double)(int16_t)y;
    }
    const uint32_t x = __byte_perm(reinterpret_cast<const uint32_t *>(g)[k], 0u, 0x0123);
    if (bitpix == -32) {
        *fval = __uint_as_float(x);
        return (double)*fval;
    }
    return (double)(int32_t)x;
}

// value = bscale * word + bzero in double, stored as REAL; an IEEE word with the identity
// scaling is copied as it is (fts/fti.c:101-104)
__device__ __forceinline__ float word_val(const uint8_t *g, int k, int ws, int bitpix, double s, double z, int id) {
    float f = 0.f;
    const double x = word_raw(g, k, ws, bitpix, &f);
    if (bitpix == -32 && id) return f;
    return (float)__dadd_rn(__dmul_rn(s, x), z);  // two roundings, as fticr_ (no FMA)
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
__device__ __forceinline__ float2 chalf(float2 a) { return make_float2(__fmul_rn(0.5f, a.x), __fmul_rn(0.5f, a.y)); }
// -0.5 * J * d with J = (0, 1): the complex product (-0.0, -0.5) * d (vis/visconvs.f:65)
__device__ __forceinline__ float2 cmjhalf(float2 d) {
    const float a = -0.0f, b = -0.5f;
    return make_float2(__fsub_rn(__fmul_rn(a, d.x), __fmul_rn(b, d.y)),
                       __fadd_rn(__fmul_rn(a, d.y), __fmul_rn(b, d.x)));
}

__global__ void k_uvfits_decode(const uint8_t *__restrict__ buf, int64_t n, UvDecode p, float *u, float *v,
                                float *w, float2 *vis, float *wt) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint8_t *g = buf + t * (int64_t)p.lgrp * p.ws;
    float pv[4];
#pragma unroll
    for (int j = 0; j < 4; j++)
        pv[j] = p.par[j] >= 0 ? word_val(g, p.par[j], p.ws, p.bitpix, p.ps[j], p.pz[j], p.pid[j]) : 0.f;
    // ARRSCALE(x, SNGL(FREQ), 0.0): OUT = SCALE * IN + OFFSET in REAL (pix/pixrscal.f)
    if (p.scale_uvw) {
#pragma unroll
        for (int j = 0; j < 3; j++) pv[j] = __fadd_rn(__fmul_rn(p.freq, pv[j]), 0.0f);
    }
    u[t] = pv[0];
    v[t] = pv[1];
    w[t] = pv[2];
    auto a = [&](int k) { return word_val(g, p.npar + k, p.ws, p.bitpix, p.bscale, p.bzero, p.aid); };
    float2 out = make_float2(0.f, 0.f);
    float ow = 0.f;
    if (p.conv == CONV_AIPS4 || p.conv == CONV_AIPS2) {
        // vis/visconvs.f:43-82, vis/visconv2.f:40-60: the pair (RR, LL) gives I and V, the pair
        // (RL, LR) gives Q and U; a pair with a non-positive weight gives 0 and weight -1
        const int b = p.pos < 2 ? 0 : 6;
        const float2 s1 = make_float2(a(b), a(b + 1)), s2 = make_float2(a(b + 3), a(b + 4));
        const float w1 = fmaxf(a(b + 2), 0.f), w2 = fmaxf(a(b + 5), 0.f);
        if (w1 > 0.f && w2 > 0.f) {
            ow = __fdiv_rn(__fadd_rn(w1, w2), 2.0f);
            if (p.pos == 0) out = chalf(cadd(s1, s2));
            else if (p.pos == 1) out = chalf(csub(s1, s2));
            else if (p.pos == 2) out = chalf(cadd(s1, s2));
            else out = cmjhalf(csub(s1, s2));
        } else {
            ow = -1.0f;
        }
    } else if (p.conv == CONV_PIPE4) {
        // vis/visconvp.f:44-80: one weight (the WEIGHT parameter) for all four; the stored WT
        // is that parameter as read (vis/visstd.f:302-304)
        const float wrr = fmaxf(pv[3], 0.f);
        if (wrr > 0.f) {
            const int b = p.pos < 2 ? 0 : 4;
            const float2 s1 = make_float2(a(b), a(b + 1)), s2 = make_float2(a(b + 2), a(b + 3));
            if (p.pos == 0) out = chalf(cadd(s1, s2));
            else if (p.pos == 1) out = chalf(csub(s1, s2));
            else if (p.pos == 2) out = chalf(cadd(s1, s2));
            else out = cmjhalf(csub(s1, s2));
        }
        ow = pv[3];
    } else {
        // no conversion: the Stokes plane at that position (vis/visstd.f:265-301)
        const int b = p.inc * p.pos;
        out = make_float2(a(b), a(b + 1));
        ow = p.inc == 3 ? a(b + 2) : pv[3];
    }
    vis[t] = out;
    wt[t] = ow;
}

int fail(const char *msg) {
    sde_set_error("%s", msg);
    return SDE_EINVAL;
}

}  // namespace

extern "C" int sde_uvfits_open(const char *path, sde_uvfits **out) {
    if (!path || !out) return fail("sde_uvfits_open: bad arguments");
    *out = nullptr;
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        sde_set_error("sde_uvfits_open: cannot open %s", path);
        return SDE_EINVAL;
    }
    Header h;
    int64_t off = 0;
    int rc = read_header(fp, &h, &off);
    fseek(fp, 0, SEEK_END);
    const int64_t fsize = (int64_t)ftell(fp);
    fclose(fp);
    if (rc != SDE_OK) return rc;
    // fts/ftsgrpre.f:64-90
    if (!h.logical("GROUPS")) return fail("Not a groups file");
    double gc = 0, pc = 0, bp = 0, nax = 0;
    if (!h.num("GCOUNT", &gc) || gc < 1) return fail("No groups!");
    if (!h.num("PCOUNT", &pc) || pc < 0 || pc > 999) return fail("sde_uvfits_open: bad PCOUNT");
    if (!h.num("BITPIX", &bp)) return fail("sde_uvfits_open: no BITPIX");
    const int bitpix = (int)bp;
    // fts/ftsgrpre.f:191-200: 16- and 32-bit integers, IEEE single
    if (bitpix != 16 && bitpix != 32 && bitpix != -32) {
        sde_set_error("Cannot read %d-bit files", bitpix);
        return SDE_EINVAL;
    }
    if (!h.num("NAXIS", &nax) || nax < 3 || nax > 16) return fail("sde_uvfits_open: bad NAXIS");
    auto sde = std::unique_ptr<sde_uvfits>(new sde_uvfits());
    sde_uvfits *f = sde.get();
    f->path = path;
    f->data_off = off;
    f->d.ngroups = (int64_t)gc;
    f->d.npar = (int)pc;
    f->d.bitpix = bitpix;
    f->ws = bitpix == 16 ? 2 : 4;
    f->bscale = h.num_or("BSCALE", 1.0);
    f->bzero = h.num_or("BZERO", 0.0);
    // array axes: NAXIS2.. (NAXIS1 = 0 marks random groups); vis/visstd.f:102-131
    int nreg = 1, stokes_ax = -1;
    double freq = 0.0;
    bool have_freq = false;
    for (int k = 2; k <= (int)nax; k++) {
        const std::string ks = std::to_string(k);
        double nk = 0;
        if (!h.num("NAXIS" + ks, &nk) || nk < 1) return fail("sde_uvfits_open: bad NAXISn");
        nreg *= (int)nk;
        const std::string ct = h.str("CTYPE" + ks);
        if (k == 2) {
            if (ct != "COMPLEX") return fail("First axis not COMPLEX");
            f->d.ncomplex = (int)nk;
        }
        if (ct == "STOKES" && stokes_ax < 0) {
            stokes_ax = k;
            f->d.nstokes = (int)nk;
            f->d.iquv = h.num_or("CRVAL" + ks, 0.0) > 0.0;
        }
        if (ct == "FREQ") {
            // FREQ = RVAL + (1.0 - RPIX) * DELT, RPIX and DELT REAL (vis/visstd.f:125)
            const float rpix = (float)h.num_or("CRPIX" + ks, 0.0), delt = (float)h.num_or("CDELT" + ks, 0.0);
            freq = h.num_or("CRVAL" + ks, 0.0) + (double)((1.0f - rpix) * delt);
            have_freq = true;
        }
        if (ct.compare(0, 2, "RA") == 0) f->d.ra = h.num_or("CRVAL" + ks, 0.0);
        if (ct.compare(0, 3, "DEC") == 0) f->d.dec = h.num_or("CRVAL" + ks, 0.0);
    }
    if (stokes_ax < 0) return fail("No stokes axes");
    if (!have_freq || freq == 0.0) return fail("No frequency");
    f->d.freq = freq;
    f->nreg = nreg;
    f->lgrp = f->d.npar + nreg;
    // random parameters (fts/ftsgrpre.f:98-148): the first of each name
    std::vector<std::string> names((size_t)f->d.npar);
    f->pscal.assign((size_t)f->d.npar, 1.0);
    f->pzero.assign((size_t)f->d.npar, 0.0);
    for (int k = 0; k < f->d.npar; k++) {
        const std::string ks = std::to_string(k + 1);
        names[(size_t)k] = h.str("PTYPE" + ks);
        f->pscal[(size_t)k] = h.num_or("PSCAL" + ks, 1.0);
        f->pzero[(size_t)k] = h.num_or("PZERO" + ks, 0.0);
    }
    auto find = [&](const char *nm) {
        for (int k = 0; k < f->d.npar; k++)
            if (names[(size_t)k] == nm) return k;
        return -1;
    };
    // vis/visstd.f:135-202: UU, UU--, UU---SIN, UU  -SIN are in seconds (scaled by SNGL(FREQ));
    // UU-L-SIN, UU-L already in wavelengths
    const char *scaled[] = {"", "--", "---SIN", "  -SIN"}, *wl[] = {"-L-SIN", "-L"};
    int *slot[3] = {&f->par_u, &f->par_v, &f->par_w};
    const char *axis[3] = {"UU", "VV", "WW"};
    int kinds[3] = {-1, -1, -1};
    for (int a = 0; a < 3; a++) {
        for (const char *sfx : scaled) {
            if (*slot[a] >= 0) break;
            *slot[a] = find((std::string(axis[a]) + sfx).c_str());
            if (*slot[a] >= 0) kinds[a] = 1;
        }
        for (const char *sfx : wl) {
            if (*slot[a] >= 0) break;
            *slot[a] = find((std::string(axis[a]) + sfx).c_str());
            if (*slot[a] >= 0) kinds[a] = 0;
        }
        if (*slot[a] < 0) {
            sde_set_error("PTYPE=%s not in header", axis[a]);
            return SDE_EINVAL;
        }
    }
    if (kinds[0] != kinds[1] || kinds[0] != kinds[2])
        return fail("sde_uvfits_open: UU, VV and WW in different units");
    f->d.uvw_scaled = kinds[0];
    // vis/visstd.f:225-258: AIPS form (re, im, wt) or pipeline form (re, im + WEIGHT)
    if (f->d.ncomplex != 3 && f->d.ncomplex != 2) return fail("Unable to read such data");
    if (f->d.ncomplex == 2) {
        f->par_wt = find("WEIGHT");
        if (f->par_wt < 0) return fail("sde_uvfits_open: pipeline-form data without a WEIGHT parameter");
    }
    // the Stokes conversions take a group as exactly one COMPLEX x STOKES block
    if (nreg != f->d.ncomplex * f->d.nstokes)
        return fail("sde_uvfits_open: more than one frequency channel, IF or position per group");
    const int64_t avail = fsize > off ? (fsize - off) / ((int64_t)f->lgrp * f->ws) : 0;
    f->d.ngroups_in_file = avail < f->d.ngroups ? avail : f->d.ngroups;
    *out = sde.release();
    return SDE_OK;
}

extern "C" int sde_uvfits_describe(const sde_uvfits *f, sde_uvfits_desc *d) {
    if (!f || !d) return fail("sde_uvfits_describe: bad arguments");
    *d = f->d;
    return SDE_OK;
}

extern "C" int sde_uvfits_close(sde_uvfits *f) {
    delete f;
    return SDE_OK;
}

extern "C" int sde_uvfits_read(sde_ctx *ctx, const sde_uvfits *f, int stokes, float *u, float *v, float *w,
                               float *vis, float *wt, int where, int64_t *nread) {
    if (!ctx || !f || !u || !v || !w || !vis || !wt || (where != SDE_HOST && where != SDE_DEVICE))
        return fail("sde_uvfits_read: bad arguments");
    // the Stokes order after conversion (vis/visstd.f:88 STKTYPE = I, V, Q, U)
    const char *order = "IVQU";
    const char *hit = stokes ? strchr(order, stokes) : nullptr;
    if (!hit) return fail("sde_uvfits_read: Stokes must be one of I, V, Q, U");
    const int pos = (int)(hit - order);
    UvDecode p{};
    p.lgrp = f->lgrp;
    p.ws = f->ws;
    p.bitpix = f->d.bitpix;
    p.npar = f->d.npar;
    p.inc = f->d.ncomplex;
    p.pos = pos;
    const int ns = f->d.nstokes;
    if (f->d.ncomplex == 3 && ns == 4 && !f->d.iquv) p.conv = CONV_AIPS4;
    else if (f->d.ncomplex == 3 && ns == 2 && !f->d.iquv) p.conv = CONV_AIPS2;
    else if (f->d.ncomplex == 2 && ns == 4) p.conv = CONV_PIPE4;
    else p.conv = CONV_NONE;
    if (pos >= ns) {
        sde_set_error("sde_uvfits_read: Stokes %c not in the file (%d Stokes planes)", stokes, ns);
        return SDE_EINVAL;
    }
    const int pars[4] = {f->par_u, f->par_v, f->par_w, f->par_wt};
    for (int j = 0; j < 4; j++) {
        p.par[j] = pars[j];
        p.ps[j] = pars[j] >= 0 ? f->pscal[(size_t)pars[j]] : 1.0;
        p.pz[j] = pars[j] >= 0 ? f->pzero[(size_t)pars[j]] : 0.0;
        p.pid[j] = p.ps[j] == 1.0 && p.pz[j] == 0.0;
    }
    p.bscale = f->bscale;
    p.bzero = f->bzero;
    p.aid = f->bscale == 1.0 && f->bzero == 0.0;
    p.freq = (float)f->d.freq;
    p.scale_uvw = f->d.uvw_scaled;
    SDE_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t ng = f->d.ngroups;
    const size_t gbytes = (size_t)f->lgrp * f->ws;
    // outputs: the caller's device arrays, or device scratch copied out at the end
    float *du = u, *dv = v, *dw = w, *dwt = wt;
    float2 *dvis = reinterpret_cast<float2 *>(vis);
    if (where == SDE_HOST) {
        SDE_TRY(ctx_scratch(ctx, "uvf_u", sizeof(float) * (size_t)ng, (void **)&du));
        SDE_TRY(ctx_scratch(ctx, "uvf_v", sizeof(float) * (size_t)ng, (void **)&dv));
        SDE_TRY(ctx_scratch(ctx, "uvf_w", sizeof(float) * (size_t)ng, (void **)&dw));
        SDE_TRY(ctx_scratch(ctx, "uvf_vis", sizeof(float2) * (size_t)ng, (void **)&dvis));
        SDE_TRY(ctx_scratch(ctx, "uvf_wt", sizeof(float) * (size_t)ng, (void **)&dwt));
    }
    // chunks of whole groups, about 32 MB, two in flight
    const int64_t cg = std::max<int64_t>(1, std::min<int64_t>(ng, (int64_t)(32u << 20) / (int64_t)gbytes));
    const size_t cbytes = (size_t)cg * gbytes;
    uint8_t *dbuf[2];
    SDE_TRY(ctx_scratch(ctx, "uvf_chunk0", cbytes, (void **)&dbuf[0]));
    SDE_TRY(ctx_scratch(ctx, "uvf_chunk1", cbytes, (void **)&dbuf[1]));
    uint8_t *hbuf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int fd = -1;
    std::unique_ptr<ChunkReader> rd;
    int rc = SDE_OK;
    int64_t done = 0;
    cudaError_t e = cudaHostAlloc((void **)&hbuf[0], cbytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&hbuf[1], cbytes, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        sde_set_error("sde_uvfits_read: %s", cudaGetErrorString(e));
        rc = SDE_ECUDA;
    }
    if (rc == SDE_OK) {
        fd = open(f->path.c_str(), O_RDONLY);
        if (fd < 0) {
            sde_set_error("sde_uvfits_read: cannot read %s", f->path.c_str());
            rc = SDE_EINVAL;
        }
    }
    if (rc == SDE_OK) {
        try {
            rd.reset(new ChunkReader(fd, reader_threads()));
        } catch (...) {
            sde_set_error("sde_uvfits_read: cannot start the reader threads");
            rc = SDE_EINVAL;
        }
    }
    for (int k = 0; rc == SDE_OK && done < ng; k ^= 1) {
        const int64_t want = std::min<int64_t>(cg, ng - done);
        // the buffer's previous copy has finished before the file overwrites it
        e = cudaEventSynchronize(ev[k]);
        if (e != cudaSuccess) break;
        const int64_t gotb = rd->read(hbuf[k], f->data_off + done * (int64_t)gbytes, want * (int64_t)gbytes);
        if (gotb < 0) {
            sde_set_error("sde_uvfits_read: cannot read %s", f->path.c_str());
            rc = SDE_EINVAL;
            break;
        }
        const int64_t got = gotb / (int64_t)gbytes;  // whole groups only, as fread counts them
        if (got > 0) {
            e = cudaMemcpyAsync(dbuf[k], hbuf[k], (size_t)got * gbytes, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) e = cudaEventRecord(ev[k], st);
            if (e != cudaSuccess) break;
            KTimer kt(ctx, "uvfits_decode");
            k_uvfits_decode<<<(unsigned)ceil_div(got, 256), 256, 0, st>>>(dbuf[k], got, p, du + done, dv + done,
                                                                        dw + done, dvis + done, dwt + done);
            e = cudaGetLastError();
            if (e != cudaSuccess) break;
            done += got;
        }
        if (got < want) break;  // end of file (fts/ftsgrpre.f:254-258)
    }
    if (e != cudaSuccess && rc == SDE_OK) {
        sde_set_error("sde_uvfits_read: %s", cudaGetErrorString(e));
        rc = SDE_ECUDA;
    }
    if (rc == SDE_OK && where == SDE_HOST && done > 0) {
        const cudaMemcpyKind k = cudaMemcpyDeviceToHost;
        e = cudaMemcpyAsync(u, du, sizeof(float) * (size_t)done, k, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(v, dv, sizeof(float) * (size_t)done, k, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(w, dw, sizeof(float) * (size_t)done, k, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(vis, dvis, sizeof(float2) * (size_t)done, k, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(wt, dwt, sizeof(float) * (size_t)done, k, st);
        if (e != cudaSuccess) {
            sde_set_error("sde_uvfits_read: %s", cudaGetErrorString(e));
            rc = SDE_ECUDA;
        }
    }
    // the pinned buffers are released only after the copies from them have finished
    const cudaError_t es = cudaStreamSynchronize(st);
    if (es != cudaSuccess && rc == SDE_OK) {
        sde_set_error("sde_uvfits_read: %s", cudaGetErrorString(es));
        rc = SDE_ECUDA;
    }
    rd.reset();
    if (fd >= 0) close(fd);
    for (int k = 0; k < 2; k++) {
        if (ev[k]) cudaEventDestroy(ev[k]);
        if (hbuf[k]) cudaFreeHost(hbuf[k]);
    }
    if (nread) *nread = done;
    if (rc == SDE_OK && done < ng) {
        char m[128];
        snprintf(m, sizeof m, "Could only read %8lld out of %8lld groups", (long long)done, (long long)ng);
        msgput_(m, "W", strlen(m), 1);
    }
    return rc;
}
