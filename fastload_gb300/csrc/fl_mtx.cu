// fl_mtx.cu -- MatrixMarket (.mtx) ingest on the GPU.
//
// Replaces the reference's host reader mmio_allinone (src/auxiliary.h:64-232,
// with mm_read_banner / mm_read_mtx_crd_size of src/mmio.h:142-259) and the
// host round trip of its CSR: the banner and size line are read on the host,
// the entry section is copied to the device in pinned chunks and tokenised,
// parsed and assembled into CSR there.
//
// Semantics kept from the reference:
//  * entries are whitespace-separated tokens read in file order (fscanf),
//    2 per entry for pattern, 3 for real / integer, 4 for complex; tokens
//    beyond the header's entry count are ignored;
//  * pattern values are 1.0, integer values are converted to double, complex
//    entries keep their real part;
//  * symmetric and hermitian files get every off-diagonal entry mirrored;
//    skew-symmetric files are read as stored (the reference's storage test
//    covers symmetric and hermitian only);
//  * CSR rows keep entries in file order, a mirrored entry taking the file
//    position of its original; duplicates are kept.
// Values are converted exactly as strtod ("%lg") converts them: the result
// is the correctly rounded double (ties to even), decided on the GPU by
//  1. the exact fast path when the significand fits 53 bits and the power of
//     ten is exact (<= 1e22): one correctly rounded multiply or divide;
//  2. an Eisel-Lemire style product with 128-bit powers of five (published
//     method: D. Lemire, "Number Parsing at a Gigabyte per Second", 2021),
//     whose table is generated here from exact integer arithmetic; with
//     the product's error bound (< 1 unit of its second word) every case the
//     bound cannot decide is passed on, so correctness does not rest on the
//     method's number-theoretic lemma;
//  3. an exact big-integer comparison of the decimal value with the midpoint
//     between two candidate doubles, for the undecided cases, subnormal
//     results and significands longer than 19 digits.
// Rejected with FL_ERR_ARG where the reference would read garbage or write
// out of bounds: malformed tokens, indices outside [1, m] x [1, n], fewer
// tokens than entries, dense (array) files, hexadecimal floats and NaN
// payloads.
#include <ctype.h>
#include <errno.h>
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "fl_internal.cuh"

namespace fl {
namespace {

// ------------------------------------------------ powers of five (host) --
// For q in [-342, 308]: 10^q ~= T_q * 2^P_q with T_q in [2^127, 2^128).
// q >= 0: T_q = the 128 leading bits of 5^q (exact while 5^q < 2^128,
// i.e. q <= 55); q < 0: T_q = ceil(2^(L+127) / 5^-q), L = bit length of
// 5^-q.
constexpr int kQMin = -342, kQMax = 308, kQCount = kQMax - kQMin + 1;

__device__ uint64_t g_pow5[kQCount][2];  // {high word, low word}
__device__ int g_pow5_exp[kQCount];

struct HostBig {
    std::vector<uint32_t> l;  // little-endian limbs
    int bits() const {
        for (int i = (int)l.size() - 1; i >= 0; i--)
            if (l[i]) return 32 * i + 32 - __builtin_clz(l[i]);
        return 0;
    }
    bool bit(int i) const { return (i >> 5) < (int)l.size() && ((l[i >> 5] >> (i & 31)) & 1); }
    void mul(uint32_t m) {
        uint64_t c = 0;
        for (auto &x : l) {
            uint64_t t = (uint64_t)x * m + c;
            x = (uint32_t)t;
            c = t >> 32;
        }
        if (c) l.push_back((uint32_t)c);
    }
    void shl1() {
        uint32_t c = 0;
        for (auto &x : l) {
            uint32_t n = x >> 31;
            x = (x << 1) | c;
            c = n;
        }
        if (c) l.push_back(c);
    }
    int cmp(const HostBig &o) const {
        int a = bits(), b = o.bits();
        if (a != b) return a < b ? -1 : 1;
        for (int i = (a + 31) / 32 - 1; i >= 0; i--) {
            uint32_t x = i < (int)l.size() ? l[i] : 0, y = i < (int)o.l.size() ? o.l[i] : 0;
            if (x != y) return x < y ? -1 : 1;
        }
        return 0;
    }
    void sub(const HostBig &o) {  // *this -= o, *this >= o
        int64_t br = 0;
        for (size_t i = 0; i < l.size(); i++) {
            int64_t t = (int64_t)l[i] - (i < o.l.size() ? o.l[i] : 0) - br;
            br = t < 0;
            l[i] = (uint32_t)(t + (br << 32));
        }
    }
};

void make_pow5_table(std::vector<uint64_t> &T, std::vector<int> &P) {
    T.assign(2 * kQCount, 0);
    P.assign(kQCount, 0);
    HostBig f;
    f.l = {1};
    for (int q = 0; q <= kQMax; q++) {  // f = 5^q
        const int L = f.bits();
        uint64_t hi = 0, lo = 0;
        for (int i = 0; i < 128; i++) {  // bit (127 - i) of T is bit (L - 1 - i) of 5^q
            const int src = L - 1 - i;
            const bool b = src >= 0 && f.bit(src);
            if (i < 64) hi |= (uint64_t)b << (63 - i);
            else lo |= (uint64_t)b << (127 - i);
        }
        T[2 * (q - kQMin)] = hi;
        T[2 * (q - kQMin) + 1] = lo;
        P[q - kQMin] = q + L - 128;
        f.mul(5);
    }
    HostBig d;
    d.l = {1};
    for (int k = 1; k <= -kQMin; k++) {  // d = 5^k, q = -k
        d.mul(5);
        const int L = d.bits();
        HostBig r;  // remainder of 2^(L-1) / d is 2^(L-1) itself (d > 2^(L-1))
        r.l.assign((L + 31) / 32 + 1, 0);
        r.l[(L - 1) >> 5] |= 1u << ((L - 1) & 31);
        uint64_t hi = 0, lo = 0;
        for (int i = 0; i < 128; i++) {
            r.shl1();
            const bool b = r.cmp(d) >= 0;
            if (b) r.sub(d);
            if (i < 64) hi |= (uint64_t)b << (63 - i);
            else lo |= (uint64_t)b << (127 - i);
        }
        if (r.bits()) {  // ceil
            if (++lo == 0) ++hi;
        }
        const int q = -k;
        T[2 * (q - kQMin)] = hi;
        T[2 * (q - kQMin) + 1] = lo;
        P[q - kQMin] = q - L - 127;
    }
}

std::mutex g_table_mu;
unsigned long long g_table_devices = 0;  // bit d: table uploaded on device d

int ensure_pow5_table() {
    int dev = 0;
    FL_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_table_mu);
    if (dev < 64 && ((g_table_devices >> dev) & 1)) return FL_SUCCESS;
    static std::vector<uint64_t> T;
    static std::vector<int> P;
    if (T.empty()) make_pow5_table(T, P);
    FL_CUDA(cudaMemcpyToSymbol(g_pow5, T.data(), T.size() * sizeof(uint64_t)));
    FL_CUDA(cudaMemcpyToSymbol(g_pow5_exp, P.data(), P.size() * sizeof(int)));
    if (dev < 64) g_table_devices |= 1ull << dev;
    return FL_SUCCESS;
}

// ------------------------------------------------------- token scanning --
__device__ __forceinline__ bool is_ws(unsigned char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

constexpr int kChunk = 16;  // bytes per thread when counting token starts

__global__ void k_tok_count(const unsigned char *t, long from, long to, int *cnt) {
    const long nch = (to - from + kChunk - 1) / kChunk;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < nch; c += (long)gridDim.x * blockDim.x) {
        const long a = from + c * kChunk, b = min(a + kChunk, to);
        bool prev_ws = a == 0 ? true : is_ws(t[a - 1]);
        int k = 0;
        for (long i = a; i < b; i++) {
            const bool w = is_ws(t[i]);
            k += (!w && prev_ws);
            prev_ws = w;
        }
        cnt[c] = k;
    }
}

__global__ void k_tok_emit(const unsigned char *t, long from, long to, const int *off, long base, long need,
                           long *starts) {
    const long nch = (to - from + kChunk - 1) / kChunk;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < nch; c += (long)gridDim.x * blockDim.x) {
        long idx = base + off[c];
        if (idx >= need) continue;
        const long a = from + c * kChunk, b = min(a + kChunk, to);
        bool prev_ws = a == 0 ? true : is_ws(t[a - 1]);
        for (long i = a; i < b && idx < need; i++) {
            const bool w = is_ws(t[i]);
            if (!w && prev_ws) starts[idx++] = i;
            prev_ws = w;
        }
    }
}

// ---------------------------------------------------------- integers ----
// %d: optional sign, decimal digits, nothing else; must fit 32 bits.
__device__ bool parse_int(const unsigned char *p, const unsigned char *e, long *out) {
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) neg = *p++ == '-';
    if (p >= e) return false;
    long v = 0;
    for (; p < e; p++) {
        const unsigned d = *p - '0';
        if (d > 9) return false;
        v = v * 10 + d;
        if (v > 2147483648L) return false;
    }
    v = neg ? -v : v;
    if (v > INT_MAX) return false;
    *out = v;
    return true;
}

// ------------------------------------------------------------ decimals --
struct Dec {
    uint64_t w;  // first 19 significant digits
    long q;      // value = w * 10^q when !trunc
    bool neg;
    bool trunc;  // a nonzero digit beyond the 19th
    int kind;    // 0 number, 1 infinity, 2 NaN, -1 malformed, -2 unsupported syntax
};

__device__ bool match_ci(const unsigned char *p, const unsigned char *e, const char *word) {
    for (; *word; word++, p++)
        if (p >= e || (*p | 0x20) != *word) return false;
    return p == e;
}

__device__ Dec scan_dec(const unsigned char *p, const unsigned char *e) {
    Dec d{0, 0, false, false, 0};
    if (p < e && (*p == '+' || *p == '-')) d.neg = *p++ == '-';
    if (p < e && (*p | 0x20) == 'i') {
        d.kind = (match_ci(p, e, "inf") || match_ci(p, e, "infinity")) ? 1 : -1;
        return d;
    }
    if (p < e && (*p | 0x20) == 'n') {
        if (match_ci(p, e, "nan")) d.kind = 2;
        else d.kind = (e - p > 3 && match_ci(p, p + 3, "nan") && p[3] == '(') ? -2 : -1;
        return d;
    }
    if (e - p >= 2 && p[0] == '0' && (p[1] | 0x20) == 'x') {
        d.kind = -2;
        return d;
    }
    int nd = 0;
    bool any = false, point = false, started = false;
    long q = 0;
    for (; p < e; p++) {
        const unsigned char c = *p;
        if (c == '.') {
            if (point) break;
            point = true;
            continue;
        }
        const unsigned dig = c - '0';
        if (dig > 9) break;
        any = true;
        if (!started) {
            if (dig == 0) {
                if (point) q--;
                continue;
            }
            started = true;
        }
        if (nd < 19) {
            d.w = d.w * 10 + dig;
            nd++;
            if (point) q--;
        } else {
            if (!point) q++;
            if (dig) d.trunc = true;
        }
    }
    if (!any) {
        d.kind = -1;
        return d;
    }
    if (p < e && (*p | 0x20) == 'e') {
        p++;
        bool eneg = false;
        if (p < e && (*p == '+' || *p == '-')) eneg = *p++ == '-';
        if (p >= e || (unsigned)(*p - '0') > 9) {
            d.kind = -1;
            return d;
        }
        long ev = 0;
        for (; p < e && (unsigned)(*p - '0') <= 9; p++)
            if (ev < 100000000L) ev = ev * 10 + (*p - '0');
        q += eneg ? -ev : ev;
    }
    if (p != e) d.kind = -1;
    d.q = q;
    return d;
}

__device__ const double kP10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                    1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

constexpr uint64_t kInfBits = 0x7ff0000000000000ull;
constexpr uint64_t kMaxBits = 0x7fefffffffffffffull;
constexpr uint64_t kFracMask = (1ull << 52) - 1;

// 192-bit product Z = (w << lz) * T_q; the value is Z * 2^x.
struct Prod {
    uint64_t top, mid, lo;
    int x;
};

__device__ __forceinline__ Prod el_product(uint64_t w, int q) {
    const int lz = __clzll((long long)w);
    const uint64_t wn = w << lz;
    const uint64_t th = g_pow5[q - kQMin][0], tl = g_pow5[q - kQMin][1];
    const uint64_t hi1 = __umul64hi(wn, th), lo1 = wn * th;
    const uint64_t hi2 = __umul64hi(wn, tl), lo2 = wn * tl;
    Prod r;
    r.mid = lo1 + hi2;
    r.top = hi1 + (r.mid < lo1);
    r.lo = lo2;
    r.x = g_pow5_exp[q - kQMin] - lz;
    return r;
}

// Correctly rounded |w * 10^q| (w != 0, q in range) when the product
// decides it: returns true and the bits; false when the exact path must
// decide (within the error bound of a midpoint, or a subnormal result).
__device__ bool el_decide(uint64_t w, int q, uint64_t *bits) {
    const Prod z = el_product(w, q);
    const int upper = (int)(z.top >> 63);        // Z in [2^(190+upper), 2^(191+upper))
    const int sh = upper + 9;                    // top >> sh keeps 54 bits
    int biased = 190 + upper + z.x + 1023;       // exponent field of the leading bit
    if (biased >= 2047) {
        *bits = kInfBits;
        return true;
    }
    if (biased <= 0) return false;
    const uint64_t m54 = z.top >> sh;
    const uint64_t rem = z.top & ((1ull << sh) - 1);
    const bool round = m54 & 1;
    uint64_t m53 = m54 >> 1;
    bool up;
    if (q >= 0 && q <= 55) {  // T_q exact: Z exact
        const bool sticky = rem | z.mid | z.lo;
        up = round && (sticky || (m53 & 1));
    } else {
        // |Z - Z_true| < 2^64 (one unit of z.mid): undecided when the part
        // below the rounding bit is within that distance of one half
        if (round && rem == 0 && z.mid == 0) return false;
        if (!round && rem == (1ull << sh) - 1 && z.mid == ~0ull) return false;
        up = round;
    }
    m53 += up;
    if (m53 >> 53) {
        m53 >>= 1;
        if (++biased >= 2047) {
            *bits = kInfBits;
            return true;
        }
    }
    *bits = ((uint64_t)biased << 52) | (m53 & kFracMask);
    return true;
}

// A double within a few units in the last place of |w * 10^q| (truncated
// product), as the starting point of the exact path.
__device__ uint64_t el_candidate(uint64_t w, int q) {
    if (w == 0 || q < kQMin) return 0;
    if (q > kQMax) return kMaxBits;
    const Prod z = el_product(w, q);
    const int upper = (int)(z.top >> 63);
    const int biased = 190 + upper + z.x + 1023;
    if (biased >= 2047) return kMaxBits;
    if (biased >= 1) return ((uint64_t)biased << 52) | ((z.top >> (upper + 10)) & kFracMask);
    // subnormal: the value in units of 2^-1074 is Z >> s, and biased <= 0
    // means s = -(x + 1074) >= 139, so only the top word contributes
    const int s = -(z.x + 1074);
    return s >= 192 ? 0 : z.top >> (s - 128);
}

// 0: bits decided; 1: exact path needed.
__device__ int dec_decide(const Dec &d, uint64_t *bits) {
    const uint64_t sign = d.neg ? 1ull << 63 : 0;
    if (d.kind == 1) {
        *bits = sign | kInfBits;
        return 0;
    }
    if (d.kind == 2) {
        *bits = sign | 0x7ff8000000000000ull;
        return 0;
    }
    if (d.w == 0) {
        *bits = sign;
        return 0;
    }
    if (d.q < kQMin) {  // below 10^19 * 10^-343 < 2^-1075: rounds to zero
        *bits = sign;
        return 0;
    }
    if (d.q > kQMax) {
        *bits = sign | kInfBits;
        return 0;
    }
    const int q = (int)d.q;
    if (!d.trunc) {
        if (d.w <= (1ull << 53) && q >= -22 && q <= 22) {
            const double x = (double)d.w;
            const double r = q >= 0 ? __dmul_rn(x, kP10[q]) : __ddiv_rn(x, kP10[-q]);
            *bits = sign | (uint64_t)__double_as_longlong(r);
            return 0;
        }
        uint64_t b;
        if (!el_decide(d.w, q, &b)) return 1;
        *bits = sign | b;
        return 0;
    }
    // value strictly between w*10^q and (w+1)*10^q
    uint64_t a, b;
    if (!el_decide(d.w, q, &a) || !el_decide(d.w + 1, q, &b) || a != b) return 1;
    *bits = sign | a;
    return 0;
}

// ------------------------------------------------------------ big ints --
// Exact path: compare D * 10^E (the decimal, up to kMaxDigits significant
// digits, plus a sticky flag for nonzero digits beyond them) with the
// midpoint F * 2^G between two adjacent doubles.  Limbs live in shared
// memory, one pair of numbers per thread.
constexpr int kLimbs = 112;  // 3584 bits: decimals of 768 digits against the extremes of binary64
constexpr int kMaxDigits = 768;
constexpr int kSlowThreads = 32;

struct Big {
    uint32_t *l;
    int n;
};

__device__ bool big_muladd(Big &a, uint32_t m, uint32_t add) {
    uint64_t c = add;
    for (int i = 0; i < a.n; i++) {
        const uint64_t t = (uint64_t)a.l[i] * m + c;
        a.l[i] = (uint32_t)t;
        c = t >> 32;
    }
    if (c) {
        if (a.n >= kLimbs) return false;
        a.l[a.n++] = (uint32_t)c;
    }
    return true;
}

__device__ bool big_mulpow5(Big &a, int k) {
    for (; k >= 13; k -= 13)
        if (!big_muladd(a, 1220703125u, 0)) return false;  // 5^13
    uint32_t m = 1;
    while (k-- > 0) m *= 5;
    return m == 1 || big_muladd(a, m, 0);
}

__device__ bool big_shl(Big &a, int s) {
    if (s == 0 || a.n == 0) return true;
    const int ws = s >> 5, bs = s & 31;
    const int n = a.n + ws + (bs ? 1 : 0);
    if (n > kLimbs) return false;
    for (int i = n - 1; i >= 0; i--) {
        const int src = i - ws;
        uint32_t v = 0;
        if (src >= 0 && src < a.n) v = bs ? a.l[src] << bs : a.l[src];
        if (bs && src - 1 >= 0 && src - 1 < a.n) v |= a.l[src - 1] >> (32 - bs);
        a.l[i] = v;
    }
    a.n = n;
    while (a.n && a.l[a.n - 1] == 0) a.n--;
    return true;
}

__device__ int big_cmp(const Big &a, const Big &b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    for (int i = a.n - 1; i >= 0; i--)
        if (a.l[i] != b.l[i]) return a.l[i] < b.l[i] ? -1 : 1;
    return 0;
}

// D (first kMaxDigits significant digits), E and the sticky flag of a
// well-formed finite decimal token.
__device__ bool big_digits(const unsigned char *p, const unsigned char *e, Big &a, long *E, bool *sticky) {
    a.n = 0;
    *sticky = false;
    if (p < e && (*p == '+' || *p == '-')) p++;
    int nd = 0, chunk_n = 0;
    uint32_t chunk = 0;
    bool point = false, started = false;
    long q = 0;
    for (; p < e; p++) {
        const unsigned char c = *p;
        if (c == '.') {
            point = true;
            continue;
        }
        const unsigned dig = c - '0';
        if (dig > 9) break;
        if (!started) {
            if (dig == 0) {
                if (point) q--;
                continue;
            }
            started = true;
        }
        if (nd < kMaxDigits) {
            chunk = chunk * 10 + dig;
            if (++chunk_n == 9) {
                if (!big_muladd(a, 1000000000u, chunk)) return false;
                chunk = 0;
                chunk_n = 0;
            }
            nd++;
            if (point) q--;
        } else {
            if (!point) q++;
            if (dig) *sticky = true;
        }
    }
    if (chunk_n) {
        uint32_t m = 1;
        for (int i = 0; i < chunk_n; i++) m *= 10;
        if (!big_muladd(a, m, chunk)) return false;
    }
    if (p < e && (*p | 0x20) == 'e') {
        p++;
        bool eneg = false;
        if (p < e && (*p == '+' || *p == '-')) eneg = *p++ == '-';
        long ev = 0;
        for (; p < e && (unsigned)(*p - '0') <= 9; p++)
            if (ev < 100000000L) ev = ev * 10 + (*p - '0');
        q += eneg ? -ev : ev;
    }
    *E = q;
    return true;
}

// sign of (decimal - midpoint(b, b + 1 ulp)) for positive finite bits b;
// 2 on capacity overflow.
__device__ int cmp_mid(const unsigned char *p, const unsigned char *e, uint64_t b, Big &A, Big &B) {
    const int biased = (int)(b >> 52);
    const uint64_t M = biased ? (b & kFracMask) | (1ull << 52) : b & kFracMask;
    const long G = (biased ? biased - 1075 : -1074) - 1;
    const uint64_t F = 2 * M + 1;
    long E;
    bool sticky;
    if (!big_digits(p, e, A, &E, &sticky)) return 2;
    B.n = 0;
    B.l[B.n++] = (uint32_t)F;
    B.l[B.n++] = (uint32_t)(F >> 32);
    while (B.n && B.l[B.n - 1] == 0) B.n--;
    if (E >= 0) {
        if (!big_mulpow5(A, (int)E)) return 2;
        const long s = E < G ? E : G;
        if (!big_shl(A, (int)(E - s)) || !big_shl(B, (int)(G - s))) return 2;
    } else {
        if (!big_mulpow5(B, (int)-E)) return 2;
        if (G - E >= 0) {
            if (!big_shl(B, (int)(G - E))) return 2;
        } else if (!big_shl(A, (int)(E - G))) {
            return 2;
        }
    }
    int c = big_cmp(A, B);
    if (c == 0 && sticky) c = 1;
    return c;
}

__device__ __forceinline__ const unsigned char *tok_end(const unsigned char *t, long start) {
    const unsigned char *p = t + start;
    while (!is_ws(*p)) p++;  // the buffer ends with a whitespace sentinel
    return p;
}

// ----------------------------------------------------------- entries ----
enum : int {
    E_INDEX_SYNTAX = 1,
    E_INDEX_RANGE = 2,
    E_VALUE_SYNTAX = 4,
    E_VALUE_UNSUPPORTED = 8,
    E_EXACT_PATH = 16,
};

struct EntryArgs {
    const unsigned char *text;
    const long *starts;
    int nnz, k, field, m, n;
    int *row, *col;
    double *val;
    int *slow, *nslow;
    int *err, *first_bad;
};

__device__ void entry_error(const EntryArgs &a, int e, int bit) {
    atomicOr(a.err, bit);
    atomicMin(a.first_bad, e);
}

__global__ void k_parse_entries(EntryArgs a) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < a.nnz; e += (long)gridDim.x * blockDim.x) {
        const long t0 = e * a.k;
        long r, c;
        const unsigned char *s0 = a.text + a.starts[t0], *s1 = a.text + a.starts[t0 + 1];
        if (!parse_int(s0, tok_end(a.text, a.starts[t0]), &r) || !parse_int(s1, tok_end(a.text, a.starts[t0 + 1]), &c)) {
            entry_error(a, (int)e, E_INDEX_SYNTAX);
            continue;
        }
        if (r < 1 || r > a.m || c < 1 || c > a.n) {
            entry_error(a, (int)e, E_INDEX_RANGE);
            continue;
        }
        a.row[e] = (int)r - 1;
        a.col[e] = (int)c - 1;
        double v = 1.0;
        if (a.field == FL_MTX_INTEGER) {
            long iv;
            if (!parse_int(a.text + a.starts[t0 + 2], tok_end(a.text, a.starts[t0 + 2]), &iv)) {
                entry_error(a, (int)e, E_VALUE_SYNTAX);
                continue;
            }
            v = (double)iv;
        } else if (a.field == FL_MTX_REAL || a.field == FL_MTX_COMPLEX) {
            const Dec d = scan_dec(a.text + a.starts[t0 + 2], tok_end(a.text, a.starts[t0 + 2]));
            if (d.kind < 0) {
                entry_error(a, (int)e, d.kind == -2 ? E_VALUE_UNSUPPORTED : E_VALUE_SYNTAX);
                continue;
            }
            if (a.field == FL_MTX_COMPLEX) {  // the imaginary part must be a number too
                const Dec im = scan_dec(a.text + a.starts[t0 + 3], tok_end(a.text, a.starts[t0 + 3]));
                if (im.kind < 0) {
                    entry_error(a, (int)e, im.kind == -2 ? E_VALUE_UNSUPPORTED : E_VALUE_SYNTAX);
                    continue;
                }
            }
            uint64_t bits;
            if (dec_decide(d, &bits)) {
                a.slow[atomicAdd(a.nslow, 1)] = (int)e;
                bits = 0;
            }
            v = __longlong_as_double((long long)bits);
        }
        a.val[e] = v;
    }
}

__global__ void __launch_bounds__(kSlowThreads) k_parse_exact(const unsigned char *text, const long *starts, int k,
                                                              const int *slow, int nslow, double *val, int *err) {
    extern __shared__ uint32_t big_smem[];
    const int i = blockIdx.x * kSlowThreads + threadIdx.x;
    if (i >= nslow) return;
    Big A{big_smem + threadIdx.x * 2 * kLimbs, 0}, B{big_smem + threadIdx.x * 2 * kLimbs + kLimbs, 0};
    const int e = slow[i];
    const long st = starts[(long)e * k + 2];
    const unsigned char *p = text + st, *end = tok_end(text, st);
    const Dec d = scan_dec(p, end);
    const uint64_t sign = d.neg ? 1ull << 63 : 0;
    uint64_t b = el_candidate(d.w, (int)max(min(d.q, (long)kQMax + 1), (long)kQMin - 1));
    bool ok = false;
    for (int it = 0; it < 8; it++) {
        if (b > 0) {
            const int c = cmp_mid(p, end, b - 1, A, B);
            if (c == 2) break;
            if (c < 0 || (c == 0 && (b & 1))) {
                b--;
                continue;
            }
        }
        if (b < kInfBits) {
            const int c = cmp_mid(p, end, b, A, B);
            if (c == 2) break;
            if (c > 0 || (c == 0 && (b & 1))) {
                b++;
                continue;
            }
        }
        ok = true;
        break;
    }
    if (!ok) {
        atomicOr(err, E_EXACT_PATH);
        return;
    }
    val[e] = __longlong_as_double((long long)(sign | b));
}

// ------------------------------------------------------------- CSR ------
__global__ void k_expand_count(const int *row, const int *col, int nnz, int sym, int *cnt,
                               unsigned long long *ndiag) {
    unsigned long long local = 0;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nnz; e += (long)gridDim.x * blockDim.x) {
        const bool off = row[e] != col[e];
        cnt[e] = (sym && off) ? 2 : 1;
        local += !off;
    }
    if (local) atomicAdd(ndiag, local);
}

__global__ void k_expand(const int *row, const int *col, const double *val, const int *pos, int nnz, int sym,
                         unsigned *key, unsigned *idx, int *ecol, double *eval, int *rowcnt) {
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nnz; e += (long)gridDim.x * blockDim.x) {
        const int p = pos[e], r = row[e], c = col[e];
        const double v = val[e];
        key[p] = r;
        idx[p] = p;
        ecol[p] = c;
        eval[p] = v;
        atomicAdd(rowcnt + r, 1);
        if (sym && r != c) {
            key[p + 1] = c;
            idx[p + 1] = p + 1;
            ecol[p + 1] = r;
            eval[p + 1] = v;
            atomicAdd(rowcnt + c, 1);
        }
    }
}

__global__ void k_csr_gather(const unsigned *idx, long nnz, const int *ecol, const double *eval, int *colidx,
                             double *val) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nnz; i += (long)gridDim.x * blockDim.x) {
        const unsigned p = idx[i];
        colidx[i] = ecol[p];
        val[i] = eval[p];
    }
}

int grid_n(long n, int threads = 256) {
    return (int)std::max<long>(1, std::min<long>((n + threads - 1) / threads, (long)num_sms() * 8));
}

int bit_length(unsigned long v) {
    int b = 0;
    while (v) {
        b++;
        v >>= 1;
    }
    return b;
}

// ------------------------------------------------------ host: header ----
struct Header {
    int field = 0, symmetry = 0;
    int m = 0, n = 0, nnz = 0;
    long data_offset = 0;
};

bool read_line(FILE *f, std::string &line) {
    line.clear();
    int c;
    while ((c = fgetc(f)) != EOF) {
        line.push_back((char)c);
        if (c == '\n') break;
    }
    return !line.empty();
}

std::vector<std::string> split_ws(const std::string &s) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && isspace((unsigned char)s[i])) i++;
        size_t j = i;
        while (j < s.size() && !isspace((unsigned char)s[j])) j++;
        if (j > i) out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

bool to_int(const std::string &s, long *v) {
    if (s.empty()) return false;
    char *end = nullptr;
    errno = 0;
    const long x = strtol(s.c_str(), &end, 10);
    if (*end || errno) return false;
    *v = x;
    return true;
}

int read_header(FILE *f, const char *path, Header *h) {
    std::string line;
    if (!read_line(f, line)) return fail(FL_ERR_IO, "mtx: %s is empty", path);
    auto tok = split_ws(line);
    if (tok.size() < 5) return fail(FL_ERR_ARG, "mtx: %s: banner needs 5 fields", path);
    if (tok[0].compare(0, 14, "%%MatrixMarket") != 0)
        return fail(FL_ERR_ARG, "mtx: %s: no %%%%MatrixMarket banner", path);
    for (int i = 1; i < 5; i++)
        for (auto &ch : tok[i]) ch = (char)tolower((unsigned char)ch);
    if (tok[1] != "matrix") return fail(FL_ERR_ARG, "mtx: %s: object '%s' is not 'matrix'", path, tok[1].c_str());
    if (tok[2] == "array") return fail(FL_ERR_ARG, "mtx: %s: dense array files are not supported", path);
    if (tok[2] != "coordinate") return fail(FL_ERR_ARG, "mtx: %s: format '%s'", path, tok[2].c_str());
    if (tok[3] == "real") h->field = FL_MTX_REAL;
    else if (tok[3] == "integer") h->field = FL_MTX_INTEGER;
    else if (tok[3] == "pattern") h->field = FL_MTX_PATTERN;
    else if (tok[3] == "complex") h->field = FL_MTX_COMPLEX;
    else return fail(FL_ERR_ARG, "mtx: %s: data type '%s'", path, tok[3].c_str());
    if (tok[4] == "general") h->symmetry = FL_MTX_GENERAL;
    else if (tok[4] == "symmetric") h->symmetry = FL_MTX_SYMMETRIC;
    else if (tok[4] == "hermitian") h->symmetry = FL_MTX_HERMITIAN;
    else if (tok[4] == "skew-symmetric") h->symmetry = FL_MTX_SKEW;
    else return fail(FL_ERR_ARG, "mtx: %s: storage scheme '%s'", path, tok[4].c_str());
    // comments, then the size line "M N nnz" (further lines if it is blank)
    do {
        if (!read_line(f, line)) return fail(FL_ERR_ARG, "mtx: %s: no size line", path);
    } while (line[0] == '%');
    long v[3];
    int got = 0;
    while (true) {
        for (const auto &t : split_ws(line)) {
            if (got == 3) break;
            if (!to_int(t, &v[got])) return fail(FL_ERR_ARG, "mtx: %s: bad size line", path);
            got++;
        }
        if (got == 3) break;
        if (got > 0 || !read_line(f, line)) return fail(FL_ERR_ARG, "mtx: %s: bad size line", path);
    }
    if (v[0] < 0 || v[1] < 0 || v[2] < 0 || v[0] > INT_MAX || v[1] > INT_MAX || v[2] > INT_MAX)
        return fail(FL_ERR_ARG, "mtx: %s: sizes %ld x %ld with %ld entries", path, v[0], v[1], v[2]);
    h->m = (int)v[0];
    h->n = (int)v[1];
    h->nnz = (int)v[2];
    h->data_offset = ftell(f);
    return FL_SUCCESS;
}

struct HostPinned {
    void *p = nullptr;
    ~HostPinned() { if (p) cudaFreeHost(p); }
};

struct Events {
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Events() { for (auto x : e) if (x) cudaEventDestroy(x); }
};

// file bytes [off, off+len) -> device buffer, in pinned chunks
int upload_file(FILE *f, const char *path, long off, long len, unsigned char *dst, cudaStream_t s) {
    if (len == 0) return FL_SUCCESS;
    const long kPiece = 32L << 20;
    const long piece = std::min(len, kPiece);
    HostPinned buf[2];
    Events ev;
    for (int i = 0; i < 2; i++) {
        FL_CUDA(cudaHostAlloc(&buf[i].p, piece, cudaHostAllocDefault));
        FL_CUDA(cudaEventCreateWithFlags(&ev.e[i], cudaEventDisableTiming));
    }
    if (fseek(f, off, SEEK_SET) != 0) return fail(FL_ERR_IO, "mtx: cannot seek in %s", path);
    bool used[2] = {false, false};
    for (long done = 0, i = 0; done < len; i++) {
        const int b = (int)(i & 1);
        if (used[b]) FL_CUDA(cudaEventSynchronize(ev.e[b]));
        const long want = std::min(piece, len - done);
        if ((long)fread(buf[b].p, 1, want, f) != want) return fail(FL_ERR_IO, "mtx: %s: read failed", path);
        FL_CUDA(cudaMemcpyAsync(dst + done, buf[b].p, want, cudaMemcpyHostToDevice, s));
        FL_CUDA(cudaEventRecord(ev.e[b], s));
        used[b] = true;
        done += want;
    }
    FL_CUDA(cudaStreamSynchronize(s));
    return FL_SUCCESS;
}

}  // namespace
}  // namespace fl

struct fl_mtx {
    fl_mtx_info info;
    fl::DevBuf<int> rowptr, colidx;
    fl::DevBuf<double> val;
};

using namespace fl;

extern "C" int fl_mtx_read(fl_mtx_t *out, const char *path, void *stream) {
    clear_error();
    if (!out || !path) return fail(FL_ERR_ARG, "mtx_read: NULL argument");
    *out = nullptr;
    const cudaStream_t s = (cudaStream_t)stream;
    FILE *f = fopen(path, "rb");
    if (!f) return fail(FL_ERR_IO, "mtx: cannot open %s", path);
    std::unique_ptr<FILE, int (*)(FILE *)> guard(f, fclose);
    Header h;
    FL_TRY(read_header(f, path, &h));
    if (fseek(f, 0, SEEK_END) != 0) return fail(FL_ERR_IO, "mtx: cannot seek in %s", path);
    const long file_bytes = ftell(f);
    const long len = file_bytes - h.data_offset;
    std::unique_ptr<fl_mtx> M(new (std::nothrow) fl_mtx());
    if (!M) return fail(FL_ERR_ALLOC, "mtx: host allocation failed");
    fl_mtx_info &I = M->info;
    memset(&I, 0, sizeof I);
    I.m = h.m;
    I.n = h.n;
    I.nnz_file = h.nnz;
    I.field = h.field;
    I.symmetry = h.symmetry;
    I.is_symmetric = h.symmetry == FL_MTX_SYMMETRIC || h.symmetry == FL_MTX_HERMITIAN;
    I.file_bytes = (size_t)file_bytes;
    if (I.is_symmetric && h.m != h.n)  // mirrored entries would fall outside the matrix
        return fail(FL_ERR_ARG, "mtx: %s: symmetric storage of a %d x %d matrix", path, h.m, h.n);
    const int k = h.field == FL_MTX_PATTERN ? 2 : h.field == FL_MTX_COMPLEX ? 4 : 3;
    const long need = (long)h.nnz * k;
    FL_TRY(ensure_pow5_table());

    // text -> device (plus a whitespace sentinel), token starts
    DevBuf<unsigned char> text;
    FL_TRY(text.alloc(len + 1, s));
    FL_TRY(upload_file(f, path, h.data_offset, len, text.get(), s));
    FL_CUDA(cudaMemsetAsync(text.get() + len, '\n', 1, s));
    DevBuf<long> starts;
    FL_TRY(starts.alloc(std::max(need, 1L), s));
    long ntok = 0;
    {
        const long kSeg = 1L << 30;  // token counts of a segment fit an int scan
        DevBuf<int> cnt;
        FL_TRY(cnt.alloc(std::max(1L, (std::min(len, kSeg) + kChunk - 1) / kChunk + 1), s));
        for (long from = 0; from < len && ntok < need; from += kSeg) {
            const long to = std::min(len, from + kSeg), nch = (to - from + kChunk - 1) / kChunk;
            k_tok_count<<<grid_n(nch), 256, 0, s>>>(text.get(), from, to, cnt.get());
            FL_CUDA(cudaGetLastError());
            FL_TRY(scan_exclusive(cnt.get(), cnt.get(), nch, cnt.get() + nch, s));
            k_tok_emit<<<grid_n(nch), 256, 0, s>>>(text.get(), from, to, cnt.get(), ntok, need, starts.get());
            FL_CUDA(cudaGetLastError());
            int seg_tokens = 0;
            FL_CUDA(cudaMemcpyAsync(&seg_tokens, cnt.get() + nch, sizeof(int), cudaMemcpyDeviceToHost, s));
            FL_CUDA(cudaStreamSynchronize(s));
            ntok += seg_tokens;
        }
    }
    if (ntok < need)
        return fail(FL_ERR_ARG, "mtx: %s: %ld tokens for %d entries of %d fields", path, ntok, h.nnz, k);

    // entries
    DevBuf<int> row, col, slow, scal;
    DevBuf<double> val;
    const int nz = h.nnz;
    FL_TRY(row.alloc(std::max(nz, 1), s));
    FL_TRY(col.alloc(std::max(nz, 1), s));
    FL_TRY(val.alloc(std::max(nz, 1), s));
    FL_TRY(slow.alloc(std::max(nz, 1), s));
    FL_TRY(scal.alloc(4, s));  // err, first bad entry, slow count
    const int init[4] = {0, INT_MAX, 0, 0};
    FL_CUDA(cudaMemcpyAsync(scal.get(), init, sizeof init, cudaMemcpyHostToDevice, s));
    if (nz) {
        EntryArgs a{text.get(), starts.get(), nz, k, h.field, h.m, h.n, row.get(), col.get(), val.get(),
                    slow.get(), scal.get() + 2, scal.get(), scal.get() + 1};
        k_parse_entries<<<grid_n(nz), 256, 0, s>>>(a);
        FL_CUDA(cudaGetLastError());
    }
    int hs[4];
    FL_CUDA(cudaMemcpyAsync(hs, scal.get(), sizeof hs, cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    if (hs[0]) {
        const int e = hs[1];
        const char *what = (hs[0] & E_INDEX_SYNTAX) ? "malformed index"
                           : (hs[0] & E_INDEX_RANGE) ? "index out of range"
                           : (hs[0] & E_VALUE_UNSUPPORTED) ? "unsupported value syntax (hexadecimal float or NaN payload)"
                                                             : "malformed value";
        return fail(FL_ERR_ARG, "mtx: %s: %s (first bad entry %d of %d, flags 0x%x)", path, what, e + 1, nz, hs[0]);
    }
    const int nslow = hs[2];
    I.exact_path_values = nslow;
    if (nslow) {
        const int blocks = (nslow + kSlowThreads - 1) / kSlowThreads;
        const size_t smem = (size_t)kSlowThreads * 2 * kLimbs * sizeof(uint32_t);
        k_parse_exact<<<blocks, kSlowThreads, smem, s>>>(text.get(), starts.get(), k, slow.get(), nslow, val.get(),
                                                          scal.get());
        FL_CUDA(cudaGetLastError());
        FL_CUDA(cudaMemcpyAsync(hs, scal.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
        FL_CUDA(cudaStreamSynchronize(s));
        if (hs[0]) return fail(FL_ERR_INTERNAL, "mtx: %s: exact conversion exceeded its limits", path);
    }
    text.release();
    starts.release();
    slow.release();

    // CSR in the reference's order: rows in file order, mirrors at the
    // file position of their original
    const int sym = I.is_symmetric;
    DevBuf<int> cnt;
    DevBuf<unsigned long long> ndiag;
    FL_TRY(cnt.alloc((size_t)nz + 1, s));
    FL_TRY(ndiag.alloc(1, s));
    FL_CUDA(cudaMemsetAsync(ndiag.get(), 0, sizeof(unsigned long long), s));
    if (nz) {
        k_expand_count<<<grid_n(nz), 256, 0, s>>>(row.get(), col.get(), nz, sym, cnt.get(), ndiag.get());
        FL_CUDA(cudaGetLastError());
    }
    unsigned long long hd = 0;
    FL_CUDA(cudaMemcpyAsync(&hd, ndiag.get(), sizeof hd, cudaMemcpyDeviceToHost, s));
    FL_CUDA(cudaStreamSynchronize(s));
    const long total = (long)nz + (sym ? (long)nz - (long)hd : 0);
    if (total > INT_MAX) return fail(FL_ERR_OVERFLOW, "mtx: %s: %ld entries after symmetric expansion", path, total);
    I.nnz = (int)total;
    FL_TRY(scan_exclusive(cnt.get(), cnt.get(), nz, cnt.get() + nz, s));
    DevBuf<unsigned> key, idx;
    DevBuf<int> ecol, rowcnt;
    DevBuf<double> evals;
    FL_TRY(key.alloc(std::max(total, 1L), s));
    FL_TRY(idx.alloc(std::max(total, 1L), s));
    FL_TRY(ecol.alloc(std::max(total, 1L), s));
    FL_TRY(evals.alloc(std::max(total, 1L), s));
    FL_TRY(rowcnt.alloc((size_t)h.m + 1, s));
    FL_CUDA(cudaMemsetAsync(rowcnt.get(), 0, ((size_t)h.m + 1) * sizeof(int), s));
    if (nz) {
        k_expand<<<grid_n(nz), 256, 0, s>>>(row.get(), col.get(), val.get(), cnt.get(), nz, sym, key.get(), idx.get(),
                                            ecol.get(), evals.get(), rowcnt.get());
        FL_CUDA(cudaGetLastError());
    }
    row.release();
    col.release();
    val.release();
    FL_TRY(M->rowptr.alloc((size_t)h.m + 1, s));
    FL_TRY(scan_exclusive(rowcnt.get(), M->rowptr.get(), h.m, M->rowptr.get() + h.m, s));
    FL_TRY(M->colidx.alloc(std::max(total, 1L), s));
    FL_TRY(M->val.alloc(std::max(total, 1L), s));
    if (total) {
        FL_TRY(radix_sort_pairs(key.get(), idx.get(), total, bit_length((unsigned long)std::max(h.m - 1, 0)), s));
        k_csr_gather<<<grid_n(total), 256, 0, s>>>(idx.get(), total, ecol.get(), evals.get(), M->colidx.get(),
                                                    M->val.get());
        FL_CUDA(cudaGetLastError());
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(FL_ERR_CUDA, "mtx: %s", cudaGetErrorString(e));
    *out = M.release();
    return FL_SUCCESS;
}

extern "C" int fl_mtx_info_get(fl_mtx_t mtx, fl_mtx_info *info) {
    clear_error();
    if (!mtx || !info) return fail(FL_ERR_ARG, "mtx_info: NULL argument");
    *info = mtx->info;
    return FL_SUCCESS;
}

extern "C" int fl_mtx_csr(fl_mtx_t mtx, const int **d_rowptr, const int **d_colidx, const double **d_val) {
    clear_error();
    if (!mtx) return fail(FL_ERR_ARG, "mtx_csr: NULL handle");
    if (d_rowptr) *d_rowptr = mtx->rowptr.get();
    if (d_colidx) *d_colidx = mtx->colidx.get();
    if (d_val) *d_val = mtx->val.get();
    return FL_SUCCESS;
}

extern "C" int fl_mtx_copy_csr(fl_mtx_t mtx, int *d_rowptr, int *d_colidx, double *d_val, void *stream) {
    clear_error();
    if (!mtx) return fail(FL_ERR_ARG, "mtx_copy_csr: NULL handle");
    const cudaStream_t s = (cudaStream_t)stream;
    const fl_mtx_info &I = mtx->info;
    if (d_rowptr)
        FL_CUDA(cudaMemcpyAsync(d_rowptr, mtx->rowptr.get(), ((size_t)I.m + 1) * sizeof(int), cudaMemcpyDeviceToDevice, s));
    if (d_colidx && I.nnz)
        FL_CUDA(cudaMemcpyAsync(d_colidx, mtx->colidx.get(), (size_t)I.nnz * sizeof(int), cudaMemcpyDeviceToDevice, s));
    if (d_val && I.nnz)
        FL_CUDA(cudaMemcpyAsync(d_val, mtx->val.get(), (size_t)I.nnz * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return FL_SUCCESS;
}

extern "C" int fl_mtx_destroy(fl_mtx_t mtx) {
    delete mtx;
    return FL_SUCCESS;
}

extern "C" int fl_mmio_allinone(int *m, int *n, int *nnz, int *isSymmetric, int **csrrowptr, int **csrcolidx,
                                double **csrval, const char *filename) {
    clear_error();
    if (!m || !n || !nnz || !isSymmetric || !csrrowptr || !csrcolidx || !csrval || !filename)
        return fail(FL_ERR_ARG, "mmio_allinone: NULL argument");
    fl_mtx_t M = nullptr;
    FL_TRY(fl_mtx_read(&M, filename, nullptr));
    std::unique_ptr<fl_mtx> guard(M);
    const fl_mtx_info &I = M->info;
    int *rp = (int *)malloc(((size_t)I.m + 1) * sizeof(int));
    int *ci = (int *)malloc(std::max<size_t>(I.nnz, 1) * sizeof(int));
    double *v = (double *)malloc(std::max<size_t>(I.nnz, 1) * sizeof(double));
    if (!rp || !ci || !v) {
        free(rp);
        free(ci);
        free(v);
        return fail(FL_ERR_ALLOC, "mmio_allinone: host allocation failed");
    }
    cudaError_t e = cudaMemcpy(rp, M->rowptr.get(), ((size_t)I.m + 1) * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && I.nnz) e = cudaMemcpy(ci, M->colidx.get(), (size_t)I.nnz * sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && I.nnz) e = cudaMemcpy(v, M->val.get(), (size_t)I.nnz * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        free(rp);
        free(ci);
        free(v);
        return fail(FL_ERR_CUDA, "mmio_allinone: %s", cudaGetErrorString(e));
    }
    *m = I.m;
    *n = I.n;
    *nnz = I.nnz;
    *isSymmetric = I.is_symmetric;
    *csrrowptr = rp;
    *csrcolidx = ci;
    *csrval = v;
    return FL_SUCCESS;
}
