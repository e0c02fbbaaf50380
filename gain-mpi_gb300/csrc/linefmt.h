// Exact printf conversions for the line list, shared by host and device code.
//
// The reference writes each line with sprintf (BaseClasses/Output.cpp:99-111):
//   "%12.6f %8d %4d %4d <- %8d %4d %4d %16.9E "  [ "%16.9E " ]  [ "[ " (" %16.9E")* " ] " ]
// followed by fprintf's " || \n".  glibc converts a double by its exact binary value and
// rounds to the requested digit with ties to even (the default rounding mode).  The
// functions below do the same with a small big-integer: for y = m 2^e (m < 2^53) and a
// decimal scale k they form floor(2 y 10^k) exactly (multiplications first, then a right
// shift and divisions by powers of ten, each floor step recording whether a non-zero
// remainder was dropped), and round that half to even.  %E picks the exponent X from
// floor(log2 y) log10(2) and corrects it until the 1+prec digit significand lies in
// [10^prec, 10^(prec+1)) -- the exponent printf prints, which is fixed after rounding.
#pragma once
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define GAIN_HD __host__ __device__ __forceinline__
#else
#define GAIN_HD inline
#endif

namespace gain {
namespace fmt {

// 1280 bits: the largest intermediate is 2 m 10^333 (the smallest subnormal scaled to a
// 10-digit significand, about 2^1161) or 2 m 2^971 10^6 (the largest double in %f).
constexpr int kLimbs = 40;

struct Big {
    uint32_t w[kLimbs];   // little-endian base 2^32; w[n-1] != 0 unless n == 0
    int n;
};

GAIN_HD uint32_t pow10_32(int j) {
    uint32_t p = 1;
    for (int i = 0; i < j; ++i) p *= 10u;
    return p;
}

GAIN_HD void big_trim(Big& b) {
    while (b.n > 0 && b.w[b.n - 1] == 0) --b.n;
}

GAIN_HD void big_set(Big& b, uint64_t v) {
    b.w[0] = (uint32_t)v;
    b.w[1] = (uint32_t)(v >> 32);
    b.n = 2;
    big_trim(b);
}

GAIN_HD void big_mul(Big& b, uint32_t f) {
    uint64_t c = 0;
    for (int i = 0; i < b.n; ++i) {
        const uint64_t t = (uint64_t)b.w[i] * f + c;
        b.w[i] = (uint32_t)t;
        c = t >> 32;
    }
    if (c && b.n < kLimbs) b.w[b.n++] = (uint32_t)c;
}

GAIN_HD void big_shl(Big& b, int s) {
    if (b.n == 0 || s <= 0) return;
    const int L = s >> 5, r = s & 31;
    int n = b.n + L + 1;
    if (n > kLimbs) n = kLimbs;
    for (int i = n - 1; i >= 0; --i) {
        const int src = i - L;
        const uint32_t hi = (src >= 0 && src < b.n) ? b.w[src] : 0u;
        const uint32_t lo = (src >= 1 && src - 1 < b.n) ? b.w[src - 1] : 0u;
        b.w[i] = r ? (hi << r) | (lo >> (32 - r)) : hi;
    }
    b.n = n;
    big_trim(b);
}

// b >>= s; returns whether a non-zero bit was shifted out.
GAIN_HD bool big_shr(Big& b, int s) {
    if (b.n == 0 || s <= 0) return false;
    const int L = s >> 5, r = s & 31;
    if (L >= b.n) {
        b.n = 0;
        return true;
    }
    bool sticky = false;
    for (int i = 0; i < L; ++i) sticky |= b.w[i] != 0u;
    if (r) sticky |= (b.w[L] & ((1u << r) - 1u)) != 0u;
    const int n = b.n - L;
    for (int i = 0; i < n; ++i) {
        const uint32_t lo = b.w[i + L];
        const uint32_t hi = (i + L + 1 < b.n) ? b.w[i + L + 1] : 0u;
        b.w[i] = r ? (lo >> r) | (hi << (32 - r)) : lo;
    }
    b.n = n;
    big_trim(b);
    return sticky;
}

// b = floor(b / d); returns the remainder.
GAIN_HD uint32_t big_div(Big& b, uint32_t d) {
    uint64_t r = 0;
    for (int i = b.n - 1; i >= 0; --i) {
        const uint64_t cur = (r << 32) | b.w[i];
        b.w[i] = (uint32_t)(cur / d);
        r = cur % d;
    }
    big_trim(b);
    return (uint32_t)r;
}

GAIN_HD uint32_t big_div_1e9(Big& b) {
    uint64_t r = 0;
    for (int i = b.n - 1; i >= 0; --i) {
        const uint64_t cur = (r << 32) | b.w[i];
        const uint64_t q = cur / 1000000000ull;
        b.w[i] = (uint32_t)q;
        r = cur - q * 1000000000ull;
    }
    big_trim(b);
    return (uint32_t)r;
}

GAIN_HD void big_inc(Big& b) {
    for (int i = 0; i < b.n; ++i)
        if (++b.w[i] != 0u) return;
    if (b.n < kLimbs) b.w[b.n++] = 1u;
}

GAIN_HD uint64_t big_u64(const Big& b) {   // valid when b.n <= 2
    return b.n == 0 ? 0ull : (b.n == 1 ? (uint64_t)b.w[0] : ((uint64_t)b.w[1] << 32) | b.w[0]);
}

// q = y 10^k rounded to an integer, ties to even; y = m 2^e with m < 2^53.
GAIN_HD void scaled_round(uint64_t m, int e, int k, Big& q) {
    big_set(q, m << 1);
    for (int j = k; j > 0; j -= 9) big_mul(q, j >= 9 ? 1000000000u : pow10_32(j));
    bool sticky = false;
    if (e > 0)
        big_shl(q, e);
    else if (e < 0)
        sticky = big_shr(q, -e);
    for (int j = -k; j > 0; j -= 9) sticky |= (j >= 9 ? big_div_1e9(q) : big_div(q, pow10_32(j))) != 0u;
    const bool half = q.n > 0 && (q.w[0] & 1u);   // q = floor(2 y 10^k)
    big_shr(q, 1);
    if (half && (sticky || (q.n > 0 && (q.w[0] & 1u)))) big_inc(q);
}

struct Parts {
    uint64_t m;   // significand (hidden bit included)
    int e;        // value = m 2^e
    bool neg, nan, inf;
};

GAIN_HD Parts decompose(double x) {
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    Parts p;
    p.neg = (u >> 63) != 0;
    const int ex = (int)((u >> 52) & 0x7ff);
    const uint64_t frac = u & ((1ull << 52) - 1);
    p.nan = ex == 0x7ff && frac != 0;
    p.inf = ex == 0x7ff && frac == 0;
    p.m = ex ? (frac | (1ull << 52)) : frac;
    p.e = ex ? ex - 1075 : -1074;
    return p;
}

GAIN_HD int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

// Character sink: counts only when p is null, writes p[0 .. lim) at most.
struct Sink {
    char* p;
    long n;
    long lim;
    GAIN_HD void put(char c) {
        if (p && n < lim) p[n] = c;
        ++n;
    }
    GAIN_HD void puts(const char* s) {
        while (*s) put(*s++);
    }
    GAIN_HD void spaces(int k) {
        for (int i = 0; i < k; ++i) put(' ');
    }
    GAIN_HD void digits(uint64_t v, int width) {   // exactly width digits, zero-padded
        char t[20];
        for (int i = width - 1; i >= 0; --i) {
            t[i] = (char)('0' + v % 10u);
            v /= 10u;
        }
        for (int i = 0; i < width; ++i) put(t[i]);
    }
};

GAIN_HD int ndigits(uint64_t v) {
    int d = 1;
    while (v >= 10u) {
        v /= 10u;
        ++d;
    }
    return d;
}

// "%<width>d"
GAIN_HD void put_d(Sink& s, int v, int width) {
    const bool neg = v < 0;
    const uint64_t a = neg ? (uint64_t)(-(int64_t)v) : (uint64_t)v;
    const int nd = ndigits(a);
    s.spaces(width - nd - (neg ? 1 : 0));
    if (neg) s.put('-');
    s.digits(a, nd);
}

// "%<width>.<prec>E", prec <= 17
GAIN_HD void put_E(Sink& s, double x, int width, int prec) {
    const Parts p = decompose(x);
    if (p.nan || p.inf) {
        s.spaces(width - 3 - (p.neg ? 1 : 0));
        if (p.neg) s.put('-');
        s.puts(p.nan ? "NAN" : "INF");
        return;
    }
    uint64_t D = 0;
    int X = 0;
    if (p.m != 0) {
        const int e2 = p.e + 63 - clz64(p.m);   // floor(log2 |x|)
        const int t = e2 * 78913;               // 78913 / 2^18 ~ log10(2)
        X = t >= 0 ? (t >> 18) : -((-t + 262143) >> 18);
        uint64_t lo = 1;
        for (int i = 0; i < prec; ++i) lo *= 10u;
        const uint64_t hi = lo * 10u;
        for (int it = 0; it < 6; ++it) {
            Big q;
            scaled_round(p.m, p.e, prec - X, q);
            if (q.n > 2) {
                ++X;
                continue;
            }
            D = big_u64(q);
            if (D >= hi) {
                ++X;
                continue;
            }
            if (D < lo) {
                --X;
                continue;
            }
            break;
        }
    }
    uint64_t lo = 1;
    for (int i = 0; i < prec; ++i) lo *= 10u;
    const int ax = X < 0 ? -X : X;
    const int xd = ax >= 100 ? 3 : 2;
    const int len = (p.neg ? 1 : 0) + 1 + (prec ? 1 + prec : 0) + 2 + xd;
    s.spaces(width - len);
    if (p.neg) s.put('-');
    s.put((char)('0' + D / lo));
    if (prec) {
        s.put('.');
        s.digits(D % lo, prec);
    }
    s.put('E');
    s.put(X < 0 ? '-' : '+');
    s.digits((uint64_t)ax, xd);
}

// "%<width>.<prec>f", prec <= 9
GAIN_HD void put_F(Sink& s, double x, int width, int prec) {
    const Parts p = decompose(x);
    if (p.nan || p.inf) {
        s.spaces(width - 3 - (p.neg ? 1 : 0));
        if (p.neg) s.put('-');
        s.puts(p.nan ? "nan" : "inf");
        return;
    }
    Big q;
    q.n = 0;
    if (p.m != 0) scaled_round(p.m, p.e, prec, q);
    const uint32_t frac = prec ? big_div(q, pow10_32(prec)) : 0u;
    const int sign = p.neg ? 1 : 0;
    if (q.n <= 2) {   // integer part below 2^64
        const uint64_t ip = big_u64(q);
        const int nd = ndigits(ip);
        s.spaces(width - sign - nd - (prec ? 1 + prec : 0));
        if (sign) s.put('-');
        s.digits(ip, nd);
    } else {          // |x| >= 2^64: base-1e9 chunks of the integer part
        uint32_t chunk[kLimbs];
        int nc = 0;
        while (q.n > 0 && nc < kLimbs) chunk[nc++] = big_div_1e9(q);
        const int top = ndigits(chunk[nc - 1]);
        s.spaces(width - sign - (top + 9 * (nc - 1)) - (prec ? 1 + prec : 0));
        if (sign) s.put('-');
        s.digits(chunk[nc - 1], top);
        for (int i = nc - 2; i >= 0; --i) s.digits(chunk[i], 9);
    }
    if (prec) {
        s.put('.');
        s.digits(frac, prec);
    }
}

// Text lengths without converting, where the value range makes them certain; anything else
// is counted by the conversion itself, so the result always equals the converted length.
GAIN_HD int len_d(int v, int width) {
    const int n = ndigits(v < 0 ? (uint64_t)(-(int64_t)v) : (uint64_t)v) + (v < 0 ? 1 : 0);
    return n > width ? n : width;
}

// "%<width>.<prec>E": the printed exponent X lies in [floor(e2 log10 2), floor((e2+1) log10 2) + 1]
// with e2 = floor(log2 |x|), so for -325 <= e2 <= 321 it has two digits.
GAIN_HD int len_E(double x, int width, int prec) {
    const Parts p = decompose(x);
    int body = -1;
    if (p.nan || p.inf) {
        body = 3 + (p.neg ? 1 : 0);
    } else if (p.m == 0) {
        body = (p.neg ? 1 : 0) + 1 + (prec ? 1 + prec : 0) + 4;
    } else {
        const int e2 = p.e + 63 - clz64(p.m);
        if (e2 >= -325 && e2 <= 321) body = (p.neg ? 1 : 0) + 1 + (prec ? 1 + prec : 0) + 4;
    }
    if (body < 0) {
        Sink c{nullptr, 0, 0};
        put_E(c, x, 0, prec);
        body = (int)c.n;
    }
    return body > width ? body : width;
}

// "%<width>.<prec>f": rounding moves the integer part from floor(|x|) to at most one more, so
// when both have the same number of digits (and |x| < 2^53) that is the width of the text.
GAIN_HD int len_F(double x, int width, int prec) {
    const Parts p = decompose(x);
    int body = -1;
    if (p.nan || p.inf) {
        body = 3 + (p.neg ? 1 : 0);
    } else {
        const double a = x < 0 ? -x : x;
        if (a < 9007199254740992.0) {
            const uint64_t ip = (uint64_t)a;
            const int nd = ndigits(ip);
            if (ndigits(ip + 1) == nd) body = (p.neg ? 1 : 0) + nd + (prec ? 1 + prec : 0);
        }
    }
    if (body < 0) {
        Sink c{nullptr, 0, 0};
        put_F(c, x, 0, prec);
        body = (int)c.n;
    }
    return body > width ? body : width;
}

// One line of the list exactly as Output.cpp:99-111 writes it (sprintf into the buffer,
// then fprintf "%s || \n"); levels are 0-based and printed + 1, symmetries likewise.
struct LineFields {
    double nu, A, intensity;
    int indexF, jF, gammaF, indexI, jI, gammaI;
    int with_intensity;
    const double* amps;   // linestrength components (output_linestrengths), namp of them
    int namp;
};

GAIN_HD void put_line(Sink& s, const LineFields& f) {
    put_F(s, f.nu, 12, 6);
    s.put(' ');
    put_d(s, f.indexF + 1, 8);
    s.put(' ');
    put_d(s, f.jF, 4);
    s.put(' ');
    put_d(s, f.gammaF + 1, 4);
    s.puts(" <- ");
    put_d(s, f.indexI + 1, 8);
    s.put(' ');
    put_d(s, f.jI, 4);
    s.put(' ');
    put_d(s, f.gammaI + 1, 4);
    s.put(' ');
    put_E(s, f.A, 16, 9);
    s.put(' ');
    if (f.with_intensity) {
        put_E(s, f.intensity, 16, 9);
        s.put(' ');
    }
    if (f.amps && f.namp > 0) {
        s.puts("[ ");
        for (int i = 0; i < f.namp; ++i) {
            s.put(' ');
            put_E(s, f.amps[i], 16, 9);
        }
        s.puts(" ] ");
    }
    s.puts(" || \n");
}

// The length put_line writes for f.
GAIN_HD long line_len(const LineFields& f) {
    long n = len_F(f.nu, 12, 6) + 1 + len_d(f.indexF + 1, 8) + 1 + len_d(f.jF, 4) + 1 + len_d(f.gammaF + 1, 4) + 4 +
             len_d(f.indexI + 1, 8) + 1 + len_d(f.jI, 4) + 1 + len_d(f.gammaI + 1, 4) + 1 + len_E(f.A, 16, 9) + 1;
    if (f.with_intensity) n += len_E(f.intensity, 16, 9) + 1;
    if (f.amps && f.namp > 0) {
        n += 2 + 3;
        for (int i = 0; i < f.namp; ++i) n += 1 + len_E(f.amps[i], 16, 9);
    }
    return n + 5;
}

}  // namespace fmt
}  // namespace gain
