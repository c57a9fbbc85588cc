// mg_host.cpp -- host-side graph construction: MTX loader, the loader's
// dedup/compaction pipeline, synthetic generators and the MTX writer.
//
// The semantics follow read_input.cu:11-254 of the reference; the
// implementation is a multi-threaded bucket pipeline instead of the
// reference's fscanf + qsort over 12-byte structs:
//   1. parse the entries (parallel over line-aligned chunks of the file),
//   2. counting-sort the (expanded) entries by source row,
//   3. sort every row by (dst, file order) in parallel,
//   4. mark duplicates / CC-filtered edges, mark used vertices,
//   5. exclusive scans -> new vertex ids and edge slots, write the CSR.

#include "mg_internal.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>

namespace mgi {

static thread_local std::string g_err;

mg_status fail(mg_status s, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

void clear_error() { g_err.clear(); }

int host_threads(int n)
{
    if (n > 0) return n;
    unsigned hc = std::thread::hardware_concurrency();
    return hc ? (int)hc : 1;
}

bool inject_alloc_failure()
{
    static std::atomic<long> counter{0};
    static long fail_at = [] {
        const char *e = std::getenv("MG_FAIL_ALLOC_AT");
        return e ? std::atol(e) : 0L;
    }();
    if (fail_at <= 0) return false;
    return counter.fetch_add(1) + 1 == fail_at;
}

uint32_t pattern_weight(uint64_t seed, uint64_t entry)
{
    // splitmix64 finaliser; identical to the oracle's orc_pattern_weight
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (entry + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (uint32_t)(z % 64u) + 1u;
}

// Run fn(t, begin, end) on nt threads over [0, n) split in equal ranges.
static void parallel_ranges(int nt, int64_t n, const std::function<void(int, int64_t, int64_t)> &fn)
{
    if (nt <= 1 || n < 4096) { fn(0, 0, n); return; }
    std::vector<std::thread> th;
    th.reserve(nt);
    for (int t = 0; t < nt; t++) {
        int64_t b = n * t / nt, e = n * (t + 1) / nt;
        th.emplace_back([&fn, t, b, e] { fn(t, b, e); });
    }
    for (auto &x : th) x.join();
}

template <class T>
static bool try_resize(std::vector<T> &v, size_t n)
{
    if (inject_alloc_failure()) return false;
    try { v.resize(n); } catch (const std::bad_alloc &) { return false; }
    return true;
}

mg_status build_csr(const Entries &in, bool sym, bool cc, int32_t source, uint64_t seed, int nthreads,
                    mg_host_graph *out)
{
    const int nt = host_threads(nthreads);
    const int32_t nv = in.nv_decl;
    const int64_t nent = (int64_t)in.src.size();
    const int64_t m0 = nent * (sym ? 2 : 1);                      // read_input.cu:59
    if (m0 > INT32_MAX - 1) return fail(MG_ERR_RANGE, "too many entries (%lld)", (long long)m0);
    if (source < 0 || source >= nv) return fail(MG_ERR_RANGE, "source %d out of range [0,%d)", source, nv);
    const bool pattern = in.val.empty();
    auto weight_of = [&](int64_t entry) -> int32_t {
        return pattern ? (int32_t)pattern_weight(seed, (uint64_t)entry) : in.val[entry];
    };

    // ---- 2. counting sort by source row (directed entry k: file entry k>>sym)
    std::vector<int32_t> rowcnt;
    if (!try_resize(rowcnt, (size_t)nv + 1)) return fail(MG_ERR_OOM, "host allocation failed");
    {
        std::unique_ptr<std::atomic<int32_t>[]> cnt(new (std::nothrow) std::atomic<int32_t>[nv + 1]);
        if (!cnt) return fail(MG_ERR_OOM, "host allocation failed");
        for (int32_t i = 0; i <= nv; i++) cnt[i].store(0, std::memory_order_relaxed);
        parallel_ranges(nt, nent, [&](int, int64_t b, int64_t e) {
            for (int64_t i = b; i < e; i++) {
                cnt[in.src[i]].fetch_add(1, std::memory_order_relaxed);
                if (sym) cnt[in.dst[i]].fetch_add(1, std::memory_order_relaxed);
            }
        });
        int64_t run = 0;
        for (int32_t i = 0; i < nv; i++) { rowcnt[i] = (int32_t)run; run += cnt[i].load(std::memory_order_relaxed); }
        rowcnt[nv] = (int32_t)run;
    }
    // keys: (dst << 32) | directed entry index  -> per-row sort gives (dst, file order)
    std::vector<uint64_t> key;
    if (!try_resize(key, (size_t)std::max<int64_t>(m0, 1))) return fail(MG_ERR_OOM, "host allocation failed");
    {
        std::unique_ptr<std::atomic<int32_t>[]> pos(new (std::nothrow) std::atomic<int32_t>[nv + 1]);
        if (!pos) return fail(MG_ERR_OOM, "host allocation failed");
        for (int32_t i = 0; i <= nv; i++) pos[i].store(rowcnt[i], std::memory_order_relaxed);
        parallel_ranges(nt, nent, [&](int, int64_t b, int64_t e) {
            for (int64_t i = b; i < e; i++) {
                int64_t k0 = sym ? 2 * i : i;
                int32_t p = pos[in.src[i]].fetch_add(1, std::memory_order_relaxed);
                key[p] = ((uint64_t)(uint32_t)in.dst[i] << 32) | (uint64_t)k0;
                if (sym) {
                    int32_t q = pos[in.dst[i]].fetch_add(1, std::memory_order_relaxed);
                    key[q] = ((uint64_t)(uint32_t)in.src[i] << 32) | (uint64_t)(k0 + 1);
                }
            }
        });
    }
    // ---- 3. sort each row (rows are independent; dynamic chunks of rows)
    {
        std::atomic<int32_t> next{0};
        const int32_t chunk = 4096;
        auto work = [&] {
            for (;;) {
                int32_t r0 = next.fetch_add(chunk);
                if (r0 >= nv) break;
                int32_t r1 = std::min(nv, r0 + chunk);
                for (int32_t r = r0; r < r1; r++) std::sort(key.begin() + rowcnt[r], key.begin() + rowcnt[r + 1]);
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nt; t++) th.emplace_back(work);
        work();
        for (auto &x : th) x.join();
    }
    // ---- 4. keep flags (read_input.cu:100-114) and used-vertex marks.
    // The reference marks endpoints and tests duplicates from sorted index 1
    // on; sorted index 0 is always kept and never marks its endpoints.
    std::vector<uint8_t> keep, valid;
    if (!try_resize(keep, (size_t)std::max<int64_t>(m0, 1)) || !try_resize(valid, (size_t)nv + 1))
        return fail(MG_ERR_OOM, "host allocation failed");
    std::fill(valid.begin(), valid.end(), 0);
    // rows are processed in parallel; "previous entry" of the first entry of a
    // row is the last entry of the closest non-empty row before it.
    std::vector<int32_t> prev_nonempty(nv + 1, -1);
    {
        int32_t last = -1;
        for (int32_t r = 0; r < nv; r++) { prev_nonempty[r] = last; if (rowcnt[r + 1] > rowcnt[r]) last = r; }
    }
    int64_t first_sorted = -1;  // global sorted index 0
    for (int32_t r = 0; r < nv; r++) if (rowcnt[r + 1] > rowcnt[r]) { first_sorted = rowcnt[r]; break; }
    {
        std::atomic<int32_t> next{0};
        const int32_t chunk = 4096;
        auto work = [&] {
            for (;;) {
                int32_t r0 = next.fetch_add(chunk);
                if (r0 >= nv) break;
                int32_t r1 = std::min(nv, r0 + chunk);
                for (int32_t r = r0; r < r1; r++) {
                    for (int32_t p = rowcnt[r]; p < rowcnt[r + 1]; p++) {
                        int32_t d = (int32_t)(key[p] >> 32);
                        if (p == first_sorted) { keep[p] = 1; continue; }
                        // endpoints marked (benign same-value races on valid[])
                        valid[r] = 1; valid[d] = 1;
                        int32_t pd, ps;
                        if (p > rowcnt[r]) { ps = r; pd = (int32_t)(key[p - 1] >> 32); }
                        else { ps = prev_nonempty[r]; pd = (int32_t)(key[rowcnt[ps + 1] - 1] >> 32); }
                        uint8_t k = (ps == r && pd == d) ? 0 : 1;
                        if (cc && r >= d) k = 0;
                        keep[p] = k;
                    }
                }
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nt; t++) th.emplace_back(work);
        work();
        for (auto &x : th) x.join();
    }
    // ---- 5. scans: new vertex id = number of used vertices before it
    std::vector<int32_t> newid;
    if (!try_resize(newid, (size_t)nv + 1)) return fail(MG_ERR_OOM, "host allocation failed");
    {
        int32_t run = 0;
        for (int32_t i = 0; i < nv; i++) { newid[i] = run; run += valid[i]; }
        newid[nv] = run;
    }
    const int32_t nv2 = newid[nv];
    // Sorted entry 0 is kept without marking its endpoints; when an endpoint
    // is used nowhere else and lies after every used vertex its new id is nv2
    // and the reference writes past its arrays.  Reject that graph.
    if (first_sorted >= 0) {
        int32_t r0 = 0;
        while (rowcnt[r0 + 1] <= first_sorted) r0++;
        int32_t d0 = (int32_t)(key[first_sorted] >> 32);
        if (newid[r0] >= nv2 || newid[d0] >= nv2)
            return fail(MG_ERR_INVALID, "graph degenerates after vertex compaction");
    }
    // kept edges per row
    std::vector<int32_t> rowkeep;
    if (!try_resize(rowkeep, (size_t)nv + 1)) return fail(MG_ERR_OOM, "host allocation failed");
    parallel_ranges(nt, nv, [&](int, int64_t b, int64_t e) {
        for (int64_t r = b; r < e; r++) {
            int32_t c = 0;
            for (int32_t p = rowcnt[r]; p < rowcnt[r + 1]; p++) c += keep[p];
            rowkeep[r] = c;
        }
    });
    std::vector<int32_t> rowoff;
    if (!try_resize(rowoff, (size_t)nv + 1)) return fail(MG_ERR_OOM, "host allocation failed");
    {
        int32_t run = 0;
        for (int32_t i = 0; i < nv; i++) { rowoff[i] = run; run += rowkeep[i]; }
        rowoff[nv] = run;
    }
    const int32_t ne2 = rowoff[nv];
    out->nv = nv2; out->ne = ne2;
    out->start_p = newid[source];                                  // read_input.cu:130
    if (!try_resize(out->v, (size_t)nv2 + 1) || !try_resize(out->e, (size_t)std::max(ne2, 1)) ||
        !try_resize(out->ev, (size_t)std::max(ne2, 1)))
        return fail(MG_ERR_OOM, "host allocation failed");
    out->e.resize(ne2); out->ev.resize(ne2);
    // rows of unused vertices carry no kept edge except possibly sorted index 0
    // (whose endpoints may be unused); the reference then writes that edge with
    // the colliding new ids -- reproduce by writing rows in old-id order.
    std::fill(out->v.begin(), out->v.end(), 0);
    parallel_ranges(nt, nv, [&](int, int64_t b, int64_t e) {
        for (int64_t r = b; r < e; r++) {
            int32_t o = rowoff[r];
            for (int32_t p = rowcnt[r]; p < rowcnt[r + 1]; p++) {
                if (!keep[p]) continue;
                int32_t d = (int32_t)(key[p] >> 32);
                int64_t k = (int64_t)(key[p] & 0xffffffffull);
                out->e[o] = newid[d];
                out->ev[o] = weight_of(sym ? (k >> 1) : k);
                o++;
            }
        }
    });
    // CSR offsets from the (new) source id of every kept edge, as the
    // reference derives them (read_input.cu:158-171): offsets[new_src+1] =
    // end of that source's edges; gaps take the previous value.
    {
        std::vector<int32_t> endpos(nv2 + 1, 0);
        for (int32_t r = 0; r < nv; r++) if (rowkeep[r] > 0) endpos[newid[r] + 1] = rowoff[r] + rowkeep[r];
        out->tra = 0;
        for (int32_t i = 1; i < nv2; i++) {
            if (endpos[i] == 0) endpos[i] = endpos[i - 1];
            else if (endpos[i] - endpos[i - 1] >= 128) out->tra = 1;
        }
        endpos[nv2] = ne2;
        endpos[0] = 0;
        out->v.assign(endpos.begin(), endpos.end());
    }
    return MG_OK;
}

// ---------------------------------------------------------------------------
// MTX parsing
// ---------------------------------------------------------------------------
static inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }

// %d-style integer: optional sign then digits
static inline bool parse_int(const char *&p, const char *end, int32_t &out)
{
    while (p < end && is_space(*p)) p++;
    if (p >= end) return false;
    bool neg = false;
    if (*p == '+' || *p == '-') { neg = (*p == '-'); p++; }
    if (p >= end || *p < '0' || *p > '9') return false;
    int64_t v = 0;
    while (p < end && *p >= '0' && *p <= '9') { v = v * 10 + (*p - '0'); if (v > INT32_MAX) v = INT32_MAX; p++; }
    out = (int32_t)(neg ? -v : v);
    return true;
}

// %f then (int): short plain integers are exact in float, others go through strtof.
static inline bool parse_float_trunc(const char *&p, const char *end, int32_t &out)
{
    while (p < end && is_space(*p)) p++;
    if (p >= end) return false;
    const char *q = p;
    bool neg = false;
    if (*q == '+' || *q == '-') { neg = (*q == '-'); q++; }
    const char *d0 = q;
    int64_t v = 0;
    while (q < end && *q >= '0' && *q <= '9' && q - d0 < 8) { v = v * 10 + (*q - '0'); q++; }
    if (q > d0 && (q >= end || is_space(*q))) {  // plain integer of <= 7 digits
        out = (int32_t)(neg ? -v : v);
        p = q;
        return true;
    }
    char tmp[64];
    size_t n = 0;
    while (p + n < end && !is_space(p[n]) && n < sizeof(tmp) - 1) { tmp[n] = p[n]; n++; }
    tmp[n] = 0;
    char *ep = nullptr;
    errno = 0;
    float f = std::strtof(tmp, &ep);
    if (ep == tmp) return false;
    p += (ep - tmp);
    if (!(f > -2147483648.0f && f < 2147483648.0f)) return false;
    out = (int32_t)f;
    return true;
}

struct MtxHeader {
    int sflag = 0, nflag = 1;
    int32_t nv = 0, ncols = 0, nnz = 0;
    size_t body = 0;  // offset of the first entry
};

static mg_status parse_header(const char *buf, size_t len, uint32_t flags, MtxHeader &h)
{
    // banner: the first line (read_input.cu:25,31-35), up to 299 chars as fgets(buf,300)
    size_t p = 0;
    size_t eol = p;
    while (eol < len && buf[eol] != '\n') eol++;
    std::string banner(buf, std::min<size_t>(eol - p, 299));
    h.sflag = (banner.find("symmetric") != std::string::npos || banner.find("Hermitian") != std::string::npos);
    if (banner.find("pattern") != std::string::npos) h.nflag = 0;
    else if (banner.find("complex") != std::string::npos) h.nflag = -1;
    else h.nflag = 1;
    if (flags & MG_LOAD_SYM) h.sflag = 1;
    if (flags & MG_LOAD_NSYM) h.sflag = 0;
    p = (eol < len) ? eol + 1 : len;
    // skip lines containing '%' (read_input.cu:46-50)
    for (;;) {
        if (p >= len) return fail(MG_ERR_PARSE, "missing size line");
        size_t e = p;
        while (e < len && buf[e] != '\n') e++;
        if (memchr(buf + p, '%', e - p) == nullptr) break;
        p = (e < len) ? e + 1 : len;
    }
    const char *q = buf + p, *end = buf + len;
    if (!parse_int(q, end, h.nv) || !parse_int(q, end, h.ncols) || !parse_int(q, end, h.nnz))
        return fail(MG_ERR_PARSE, "malformed size line");
    if (h.nv < 0 || h.nnz < 0) return fail(MG_ERR_PARSE, "negative size");
    h.body = (size_t)(q - buf);
    return MG_OK;
}

// Sequential token-stream parse (fscanf semantics; entries may span lines).
static mg_status parse_entries_stream(const char *buf, size_t len, const MtxHeader &h, Entries &E)
{
    const char *p = buf + h.body, *end = buf + len;
    for (int64_t i = 0; i < h.nnz; i++) {
        int32_t s, d, w = 0, w2;
        if (!parse_int(p, end, s) || !parse_int(p, end, d))
            return fail(MG_ERR_PARSE, "truncated entry list at entry %lld", (long long)i);
        if (h.nflag == 1) { if (!parse_float_trunc(p, end, w)) return fail(MG_ERR_PARSE, "bad value at entry %lld", (long long)i); }
        else if (h.nflag == -1) {
            if (!parse_float_trunc(p, end, w) || !parse_float_trunc(p, end, w2))
                return fail(MG_ERR_PARSE, "bad complex value at entry %lld", (long long)i);
        }
        s--; d--;
        if (s < 0 || s >= h.nv || d < 0 || d >= h.nv)
            return fail(MG_ERR_RANGE, "A vertex id is out of range %d %d", s, d);
        E.src[i] = s; E.dst[i] = d;
        if (h.nflag != 0) E.val[i] = w;
    }
    return MG_OK;
}

// Parallel line-oriented parse; returns MG_ERR_INVALID when the layout is not
// one entry per line so the caller falls back to the stream parser.
static mg_status parse_entries_lines(const char *buf, size_t len, const MtxHeader &h, int nt, Entries &E)
{
    const char *body = buf + h.body, *end = buf + len;
    // start after the rest of the size line
    while (body < end && *body != '\n') {
        if (!is_space(*body)) return MG_ERR_INVALID;
        body++;
    }
    if (body < end) body++;
    size_t blen = (size_t)(end - body);
    nt = std::max(1, std::min(nt, (int)(blen / (1 << 20)) + 1));
    std::vector<size_t> cut(nt + 1);
    cut[0] = 0; cut[nt] = blen;
    for (int t = 1; t < nt; t++) {
        size_t c = blen * t / nt;
        while (c < blen && body[c - 1] != '\n') c++;
        cut[t] = c;
    }
    const int nvals = h.nflag == 0 ? 0 : (h.nflag == 1 ? 1 : 2);
    // pass 1: count entry lines per chunk
    std::vector<int64_t> cnt(nt + 1, 0);
    std::atomic<int> bad{0};
    auto count_chunk = [&](int t) {
        int64_t c = 0;
        const char *p = body + cut[t], *e = body + cut[t + 1];
        while (p < e) {
            const char *l = p;
            while (p < e && *p != '\n') p++;
            bool blank = true;
            for (const char *x = l; x < p; x++) if (!is_space(*x)) { blank = false; break; }
            if (!blank) c++;
            if (p < e) p++;
        }
        cnt[t + 1] = c;
    };
    {
        std::vector<std::thread> th;
        for (int t = 1; t < nt; t++) th.emplace_back(count_chunk, t);
        count_chunk(0);
        for (auto &x : th) x.join();
    }
    for (int t = 0; t < nt; t++) cnt[t + 1] += cnt[t];
    if (cnt[nt] < h.nnz) return MG_ERR_INVALID;  // fewer lines than entries: maybe multi-line layout
    std::atomic<int32_t> range_bad{0};
    std::atomic<int64_t> bad_s{0}, bad_d{0};
    auto parse_chunk = [&](int t) {
        int64_t i = cnt[t];
        const char *p = body + cut[t], *e = body + cut[t + 1];
        while (p < e && i < h.nnz) {
            const char *le = p;
            while (le < e && *le != '\n') le++;
            const char *q = p;
            int32_t s, d, w = 0, w2;
            const char *qq = q;
            while (qq < le && is_space(*qq)) qq++;
            if (qq == le) { p = le + 1; continue; }  // blank line
            if (!parse_int(q, le, s) || !parse_int(q, le, d)) { bad = 1; return; }
            if (nvals >= 1 && !parse_float_trunc(q, le, w)) { bad = 1; return; }
            if (nvals == 2 && !parse_float_trunc(q, le, w2)) { bad = 1; return; }
            while (q < le && is_space(*q)) q++;
            if (q != le) { bad = 1; return; }  // trailing tokens: not one entry per line
            s--; d--;
            if (s < 0 || s >= h.nv || d < 0 || d >= h.nv) {
                if (range_bad.exchange(1) == 0) { bad_s = s; bad_d = d; }
            }
            E.src[i] = s; E.dst[i] = d;
            if (nvals) E.val[i] = w;
            i++;
            p = le + 1;
        }
    };
    {
        std::vector<std::thread> th;
        for (int t = 1; t < nt; t++) th.emplace_back(parse_chunk, t);
        parse_chunk(0);
        for (auto &x : th) x.join();
    }
    if (bad) return MG_ERR_INVALID;
    if (range_bad)
        return fail(MG_ERR_RANGE, "A vertex id is out of range %d %d", (int)bad_s.load(), (int)bad_d.load());
    return MG_OK;
}

}  // namespace mgi

using namespace mgi;

extern "C" {

mg_status mg_load_mtx(const char *path, int32_t source, uint32_t flags, uint64_t weight_seed, int32_t nthreads,
                      mg_host_graph **out)
{
    clear_error();
    if (!path || !out) return fail(MG_ERR_INVALID, "null argument");
    *out = nullptr;
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(MG_ERR_IO, "cannot open %s", path);
    std::fseek(f, 0, SEEK_END);
    long flen = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (flen < 0) { std::fclose(f); return fail(MG_ERR_IO, "cannot size %s", path); }
    std::vector<char> buf;
    if (!try_resize(buf, (size_t)flen + 1)) { std::fclose(f); return fail(MG_ERR_OOM, "host allocation failed"); }
    size_t got = std::fread(buf.data(), 1, (size_t)flen, f);
    std::fclose(f);
    if (got != (size_t)flen) return fail(MG_ERR_IO, "short read on %s", path);
    buf[flen] = 0;

    MtxHeader h;
    mg_status s = parse_header(buf.data(), (size_t)flen, flags, h);
    if (s != MG_OK) return s;
    if (source < 0 || source >= h.nv) return fail(MG_ERR_RANGE, "source %d out of range [0,%d)", source, h.nv);
    Entries E;
    E.nv_decl = h.nv;
    if (!try_resize(E.src, (size_t)h.nnz) || !try_resize(E.dst, (size_t)h.nnz) ||
        (h.nflag != 0 && !try_resize(E.val, (size_t)h.nnz)))
        return fail(MG_ERR_OOM, "host allocation failed");
    s = parse_entries_lines(buf.data(), (size_t)flen, h, host_threads(nthreads), E);
    if (s == MG_ERR_INVALID) s = parse_entries_stream(buf.data(), (size_t)flen, h, E);
    if (s != MG_OK) return s;
    buf.clear(); buf.shrink_to_fit();

    std::unique_ptr<mg_host_graph> g(new (std::nothrow) mg_host_graph());
    if (!g) return fail(MG_ERR_OOM, "host allocation failed");
    s = build_csr(E, h.sflag != 0, (flags & MG_LOAD_CC) != 0, source, weight_seed, nthreads, g.get());
    if (s != MG_OK) return s;
    *out = g.release();
    return MG_OK;
}

mg_status mg_host_graph_from_entries(int32_t nv_decl, int64_t nentries, const int32_t *src, const int32_t *dst,
                                     const int32_t *val, int32_t source, uint32_t flags, uint64_t weight_seed,
                                     int32_t nthreads, mg_host_graph **out)
{
    clear_error();
    if (!out || nv_decl < 0 || nentries < 0 || (nentries > 0 && (!src || !dst)))
        return fail(MG_ERR_INVALID, "invalid argument");
    *out = nullptr;
    Entries E;
    E.nv_decl = nv_decl;
    if (!try_resize(E.src, (size_t)nentries) || !try_resize(E.dst, (size_t)nentries) ||
        (val && !try_resize(E.val, (size_t)nentries)))
        return fail(MG_ERR_OOM, "host allocation failed");
    for (int64_t i = 0; i < nentries; i++) {
        if (src[i] < 0 || src[i] >= nv_decl || dst[i] < 0 || dst[i] >= nv_decl)
            return fail(MG_ERR_RANGE, "A vertex id is out of range %d %d", src[i], dst[i]);
    }
    if (nentries) {
        std::memcpy(E.src.data(), src, sizeof(int32_t) * nentries);
        std::memcpy(E.dst.data(), dst, sizeof(int32_t) * nentries);
        if (val) std::memcpy(E.val.data(), val, sizeof(int32_t) * nentries);
    }
    bool sym = (flags & MG_LOAD_SYM) && !(flags & MG_LOAD_NSYM);
    std::unique_ptr<mg_host_graph> g(new (std::nothrow) mg_host_graph());
    if (!g) return fail(MG_ERR_OOM, "host allocation failed");
    mg_status s = build_csr(E, sym, (flags & MG_LOAD_CC) != 0, source, weight_seed, nthreads, g.get());
    if (s != MG_OK) return s;
    *out = g.release();
    return MG_OK;
}

mg_status mg_host_graph_from_csr(int32_t nv, int32_t ne, const int32_t *v, const int32_t *e, const int32_t *ev,
                                 int32_t start_p, mg_host_graph **out)
{
    clear_error();
    if (!out || nv < 0 || ne < 0 || !v || (ne > 0 && !e)) return fail(MG_ERR_INVALID, "invalid argument");
    *out = nullptr;
    if (v[0] != 0 || v[nv] != ne) return fail(MG_ERR_INVALID, "row offsets must start at 0 and end at ne");
    for (int32_t i = 0; i < nv; i++)
        if (v[i + 1] < v[i]) return fail(MG_ERR_INVALID, "row offsets not monotone at %d", i);
    for (int32_t i = 0; i < ne; i++)
        if (e[i] < 0 || e[i] >= nv) return fail(MG_ERR_RANGE, "column id %d out of range at %d", e[i], i);
    std::unique_ptr<mg_host_graph> g(new (std::nothrow) mg_host_graph());
    if (!g) return fail(MG_ERR_OOM, "host allocation failed");
    if (!try_resize(g->v, (size_t)nv + 1) || !try_resize(g->e, (size_t)ne) || !try_resize(g->ev, (size_t)ne))
        return fail(MG_ERR_OOM, "host allocation failed");
    std::memcpy(g->v.data(), v, sizeof(int32_t) * (nv + 1));
    if (ne) std::memcpy(g->e.data(), e, sizeof(int32_t) * ne);
    for (int32_t i = 0; i < ne; i++) g->ev[i] = ev ? ev[i] : 1;
    g->nv = nv; g->ne = ne; g->start_p = start_p;
    g->tra = 0;
    for (int32_t i = 0; i + 1 < nv; i++) if (v[i + 1] - v[i] >= 128) { g->tra = 1; break; }
    *out = g.release();
    return MG_OK;
}

mg_status mg_host_graph_view(const mg_host_graph *g, mg_csr_view *view)
{
    if (!g || !view) return fail(MG_ERR_INVALID, "null argument");
    view->nv = g->nv; view->ne = g->ne; view->start_p = g->start_p; view->tra = g->tra;
    view->csc_v = g->v.data(); view->csc_e = g->e.data(); view->csc_ev = g->ev.data();
    return MG_OK;
}

mg_status mg_write_mtx(const mg_host_graph *g, const char *path, int32_t with_weights)
{
    clear_error();
    if (!g || !path) return fail(MG_ERR_INVALID, "null argument");
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(MG_ERR_IO, "cannot open %s for writing", path);
    std::vector<char> buf(1 << 22);
    std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    std::fprintf(f, "%%%%MatrixMarket matrix coordinate %s general\n", with_weights ? "integer" : "pattern");
    std::fprintf(f, "%d %d %d\n", g->nv, g->nv, g->ne);
    char line[64];
    for (int32_t u = 0; u < g->nv; u++) {
        for (int32_t p = g->v[u]; p < g->v[u + 1]; p++) {
            int n = with_weights ? std::snprintf(line, sizeof(line), "%d %d %d\n", u + 1, g->e[p] + 1, g->ev[p])
                                 : std::snprintf(line, sizeof(line), "%d %d\n", u + 1, g->e[p] + 1);
            std::fwrite(line, 1, (size_t)n, f);
        }
    }
    bool ok = std::ferror(f) == 0;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MG_OK : fail(MG_ERR_IO, "write failed on %s", path);
}

// ---------------------------------------------------------------------------
// binary CSR cache
// ---------------------------------------------------------------------------
namespace {

const char CSR_MAGIC[8] = {'M', 'G', 'C', 'S', 'R', '0', '0', '1'};

struct CsrHeader {
    char magic[8];
    int32_t nv, ne, start_p, tra;
    uint32_t flags;  // bit 0: weights present (always set by mg_save_csr)
    uint32_t pad;
    uint64_t checksum;
};
static_assert(sizeof(CsrHeader) == 40, "header layout");

uint64_t fnv1a(uint64_t h, const void *data, size_t bytes)
{
    const unsigned char *p = static_cast<const unsigned char *>(data);
    for (size_t i = 0; i < bytes; i++) h = (h ^ p[i]) * 1099511628211ull;
    return h;
}

uint64_t csr_checksum(const mg_host_graph &g)
{
    uint64_t h = 1469598103934665603ull;
    h = fnv1a(h, g.v.data(), g.v.size() * 4);
    h = fnv1a(h, g.e.data(), g.e.size() * 4);
    h = fnv1a(h, g.ev.data(), g.ev.size() * 4);
    return h;
}

bool little_endian()
{
    const uint32_t x = 1;
    unsigned char c;
    std::memcpy(&c, &x, 1);
    return c == 1;
}

}  // namespace

mg_status mg_save_csr(const mg_host_graph *g, const char *path)
{
    clear_error();
    if (!g || !path) return fail(MG_ERR_INVALID, "null argument");
    if (!little_endian()) return fail(MG_ERR_UNSUPPORTED, "binary CSR files are little-endian");
    CsrHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, CSR_MAGIC, 8);
    hd.nv = g->nv;
    hd.ne = g->ne;
    hd.start_p = g->start_p;
    hd.tra = g->tra;
    hd.flags = 1;
    hd.checksum = csr_checksum(*g);
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(MG_ERR_IO, "cannot open %s for writing", path);
    bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1;
    ok = ok && std::fwrite(g->v.data(), 4, g->v.size(), f) == g->v.size();
    if (g->ne > 0) {
        ok = ok && std::fwrite(g->e.data(), 4, g->e.size(), f) == g->e.size();
        ok = ok && std::fwrite(g->ev.data(), 4, g->ev.size(), f) == g->ev.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MG_OK : fail(MG_ERR_IO, "write failed on %s", path);
}

mg_status mg_load_csr(const char *path, mg_host_graph **out)
{
    clear_error();
    if (!path || !out) return fail(MG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (!little_endian()) return fail(MG_ERR_UNSUPPORTED, "binary CSR files are little-endian");
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(MG_ERR_IO, "cannot open %s", path);
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, std::fclose);
    CsrHeader hd;
    if (std::fread(&hd, sizeof(hd), 1, f) != 1) return fail(MG_ERR_PARSE, "%s: truncated header", path);
    if (std::memcmp(hd.magic, CSR_MAGIC, 8) != 0) return fail(MG_ERR_PARSE, "%s: not a binary CSR file", path);
    if (hd.nv < 0 || hd.ne < 0 || hd.flags != 1 || (hd.nv == 0 && hd.ne != 0))
        return fail(MG_ERR_PARSE, "%s: bad header (nv %d, ne %d, flags %u)", path, hd.nv, hd.ne, hd.flags);
    if (std::fseek(f, 0, SEEK_END) != 0) return fail(MG_ERR_IO, "%s: seek failed", path);
    const long long size = std::ftell(f);
    const long long want = (long long)sizeof(hd) + 4ll * ((long long)hd.nv + 1) + 8ll * hd.ne;
    if (size != want) return fail(MG_ERR_PARSE, "%s: size %lld, header implies %lld", path, size, want);
    std::fseek(f, (long)sizeof(hd), SEEK_SET);
    if (inject_alloc_failure()) return fail(MG_ERR_OOM, "host allocation failed (injected)");
    std::unique_ptr<mg_host_graph> g(new mg_host_graph());
    g->nv = hd.nv;
    g->ne = hd.ne;
    g->start_p = hd.start_p;
    g->tra = hd.tra;
    try {
        g->v.resize((size_t)hd.nv + 1);
        g->e.resize((size_t)hd.ne);
        g->ev.resize((size_t)hd.ne);
    } catch (const std::bad_alloc &) {
        return fail(MG_ERR_OOM, "host allocation failed");
    }
    bool ok = std::fread(g->v.data(), 4, g->v.size(), f) == g->v.size();
    if (hd.ne > 0) {
        ok = ok && std::fread(g->e.data(), 4, g->e.size(), f) == g->e.size();
        ok = ok && std::fread(g->ev.data(), 4, g->ev.size(), f) == g->ev.size();
    }
    if (!ok) return fail(MG_ERR_PARSE, "%s: truncated arrays", path);
    if (csr_checksum(*g) != hd.checksum) return fail(MG_ERR_PARSE, "%s: checksum mismatch", path);
    if (g->v[0] != 0 || g->v[(size_t)hd.nv] != hd.ne) return fail(MG_ERR_PARSE, "%s: bad row offsets", path);
    for (int32_t u = 0; u < hd.nv; u++)
        if (g->v[(size_t)u + 1] < g->v[(size_t)u]) return fail(MG_ERR_PARSE, "%s: row offsets decrease at %d", path, u);
    for (int32_t p = 0; p < hd.ne; p++)
        if (g->e[(size_t)p] < 0 || g->e[(size_t)p] >= hd.nv)
            return fail(MG_ERR_PARSE, "%s: column id out of range at entry %d", path, p);
    if (hd.nv > 0 && (hd.start_p < 0 || hd.start_p >= hd.nv))
        return fail(MG_ERR_PARSE, "%s: start_p %d out of range", path, hd.start_p);
    *out = g.release();
    return MG_OK;
}

void mg_host_graph_free(mg_host_graph *g);  // defined with the CUDA parts (unpins)

// ---------------------------------------------------------------------------
// generators
// ---------------------------------------------------------------------------
static inline uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

mg_status mg_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                      int32_t wmin, int32_t wmax, int32_t nthreads, mg_host_graph **out)
{
    clear_error();
    if (!out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0 ||
        wmin > wmax)
        return fail(MG_ERR_INVALID, "invalid R-MAT parameters");
    *out = nullptr;
    const int64_t ndraw = (int64_t)edge_factor << scale;
    const int32_t nv = (int32_t)(1u << scale);
    if (ndraw > INT32_MAX / 2) return fail(MG_ERR_RANGE, "R-MAT too large for int32 CSR");
    const uint64_t ta = (uint64_t)(a * 4294967296.0), tb = (uint64_t)((a + b) * 4294967296.0),
                   tc = (uint64_t)((a + b + c) * 4294967296.0);
    const int nt = host_threads(nthreads);
    Entries E;
    E.nv_decl = nv;
    if (!try_resize(E.src, (size_t)ndraw) || !try_resize(E.dst, (size_t)ndraw) || !try_resize(E.val, (size_t)ndraw))
        return fail(MG_ERR_OOM, "host allocation failed");
    std::vector<int64_t> kept(nt + 1, 0);
    // each thread generates a contiguous range of draws, then drops self-loops
    // in place; draws are seeded per index so the graph does not depend on nt.
    std::vector<int64_t> lo(nt), hi(nt);
    parallel_ranges(nt, ndraw, [&](int t, int64_t b0, int64_t e0) {
        int64_t o = b0;
        for (int64_t i = b0; i < e0; i++) {
            uint64_t st = seed * 0xD1B54A32D192ED03ull + (uint64_t)i;
            uint32_t s = 0, d = 0;
            uint64_t r = 0;
            for (int l = 0; l < scale; l++) {
                if ((l & 1) == 0) r = splitmix(st);
                uint64_t x = (l & 1) ? (r >> 32) : (r & 0xffffffffull);
                uint32_t sb, db;
                if (x < ta) { sb = 0; db = 0; }
                else if (x < tb) { sb = 0; db = 1; }
                else if (x < tc) { sb = 1; db = 0; }
                else { sb = 1; db = 1; }
                s = (s << 1) | sb; d = (d << 1) | db;
            }
            if (s == d) continue;  // self-loops removed
            uint64_t wr = splitmix(st);
            E.src[o] = (int32_t)s; E.dst[o] = (int32_t)d;
            E.val[o] = wmin + (int32_t)(wr % (uint64_t)(wmax - wmin + 1));
            o++;
        }
        lo[t] = b0; hi[t] = o;
    });
    // compact the per-thread ranges
    int64_t w = 0;
    int used = (int)std::min<int64_t>(nt, ndraw < 4096 ? 1 : nt);
    for (int t = 0; t < used; t++) {
        int64_t n = hi[t] - lo[t];
        if (w != lo[t]) {
            std::memmove(&E.src[w], &E.src[lo[t]], sizeof(int32_t) * n);
            std::memmove(&E.dst[w], &E.dst[lo[t]], sizeof(int32_t) * n);
            std::memmove(&E.val[w], &E.val[lo[t]], sizeof(int32_t) * n);
        }
        w += n;
    }
    E.src.resize(w); E.dst.resize(w); E.val.resize(w);
    std::unique_ptr<mg_host_graph> g(new (std::nothrow) mg_host_graph());
    if (!g) return fail(MG_ERR_OOM, "host allocation failed");
    // source 0 must exist in the declared range; the caller picks sources
    // in the compacted id space afterwards
    mg_status s = build_csr(E, true, false, 0, seed, nthreads, g.get());
    if (s != MG_OK) return s;
    *out = g.release();
    return MG_OK;
}

mg_status mg_gen_lattice(int32_t rows, int32_t cols, double shortcut_frac, uint64_t seed, mg_host_graph **out)
{
    clear_error();
    if (!out || rows < 1 || cols < 1 || shortcut_frac < 0 || shortcut_frac > 1 ||
        (int64_t)rows * cols > (int64_t)INT32_MAX / 8)
        return fail(MG_ERR_INVALID, "invalid lattice parameters");
    *out = nullptr;
    const int32_t nv = rows * cols;
    const uint64_t thr = (uint64_t)(shortcut_frac * 18446744073709551615.0);
    Entries E;
    E.nv_decl = nv;
    E.src.reserve((size_t)nv * 2 + nv / 8); E.dst.reserve((size_t)nv * 2 + nv / 8);
    for (int32_t r = 0; r < rows; r++) {
        for (int32_t c = 0; c < cols; c++) {
            int32_t u = r * cols + c;
            if (c + 1 < cols) { E.src.push_back(u); E.dst.push_back(u + 1); }
            if (r + 1 < rows) { E.src.push_back(u); E.dst.push_back(u + cols); }
            uint64_t st = seed * 0xD1B54A32D192ED03ull + (uint64_t)u;
            if (r + 1 < rows && c + 1 < cols && splitmix(st) < thr) { E.src.push_back(u); E.dst.push_back(u + cols + 1); }
        }
    }
    E.val.assign(E.src.size(), 1);
    std::unique_ptr<mg_host_graph> g(new (std::nothrow) mg_host_graph());
    if (!g) return fail(MG_ERR_OOM, "host allocation failed");
    mg_status s = build_csr(E, true, false, 0, seed, 0, g.get());
    if (s != MG_OK) return s;
    *out = g.release();
    return MG_OK;
}

const char *mg_last_error(void) { return mgi::g_err.c_str(); }

const char *mg_status_string(mg_status s)
{
    switch (s) {
    case MG_OK: return "ok";
    case MG_ERR_IO: return "io error";
    case MG_ERR_PARSE: return "parse error";
    case MG_ERR_RANGE: return "out of range";
    case MG_ERR_OOM: return "out of memory";
    case MG_ERR_CUDA: return "cuda error";
    case MG_ERR_ITER_LIMIT: return "iteration limit";
    case MG_ERR_INVALID: return "invalid argument";
    case MG_ERR_UNSUPPORTED: return "unsupported";
    case MG_ERR_INTERNAL: return "internal inconsistency";
    default: return "unknown status";
    }
}

const char *mg_version(void) { return "multigraph-gb300 0.1 (sm_103a)"; }

}  // extern "C"
