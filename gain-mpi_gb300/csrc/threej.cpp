// Exact Wigner 3j symbols for the 3j table of the half line strength.
//
// The reference evaluates three_j (TroveFortran/fort_func.f90:7-104) through sums of
// log-factorials in floating point.  Here the Racah formula is evaluated in exact integer
// arithmetic: the square of the symbol is a rational p/q, and the result is the double
// nearest to sqrt(p/q) (one correct rounding), found by integer comparisons only.
#include <cmath>
#include <cstdint>
#include <vector>

#include "gain_internal.h"

namespace gain {
namespace {

// Non-negative arbitrary-precision integer, 32-bit limbs, little endian.
struct Big {
    std::vector<uint32_t> d;
    Big() {}
    explicit Big(uint64_t v) {
        while (v) { d.push_back((uint32_t)v); v >>= 32; }
    }
    void trim() { while (!d.empty() && d.back() == 0) d.pop_back(); }
    bool zero() const { return d.empty(); }
};

Big mul(const Big& a, const Big& b) {
    Big r;
    if (a.zero() || b.zero()) return r;
    r.d.assign(a.d.size() + b.d.size(), 0);
    for (size_t i = 0; i < a.d.size(); ++i) {
        uint64_t carry = 0;
        for (size_t j = 0; j < b.d.size(); ++j) {
            uint64_t cur = (uint64_t)a.d[i] * b.d[j] + r.d[i + j] + carry;
            r.d[i + j] = (uint32_t)cur;
            carry = cur >> 32;
        }
        size_t k = i + b.d.size();
        while (carry) {
            uint64_t cur = (uint64_t)r.d[k] + carry;
            r.d[k++] = (uint32_t)cur;
            carry = cur >> 32;
        }
    }
    r.trim();
    return r;
}

int cmp(const Big& a, const Big& b) {
    if (a.d.size() != b.d.size()) return a.d.size() < b.d.size() ? -1 : 1;
    for (size_t i = a.d.size(); i-- > 0;)
        if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
    return 0;
}

Big add(const Big& a, const Big& b) {
    Big r;
    size_t n = std::max(a.d.size(), b.d.size());
    r.d.assign(n + 1, 0);
    uint64_t carry = 0;
    for (size_t i = 0; i < n; ++i) {
        uint64_t cur = carry;
        if (i < a.d.size()) cur += a.d[i];
        if (i < b.d.size()) cur += b.d[i];
        r.d[i] = (uint32_t)cur;
        carry = cur >> 32;
    }
    r.d[n] = (uint32_t)carry;
    r.trim();
    return r;
}

// a - b, requires a >= b
Big sub(const Big& a, const Big& b) {
    Big r;
    r.d.assign(a.d.size(), 0);
    int64_t borrow = 0;
    for (size_t i = 0; i < a.d.size(); ++i) {
        int64_t cur = (int64_t)a.d[i] - borrow - (i < b.d.size() ? (int64_t)b.d[i] : 0);
        borrow = cur < 0;
        if (cur < 0) cur += ((int64_t)1 << 32);
        r.d[i] = (uint32_t)cur;
    }
    r.trim();
    return r;
}

Big shl(const Big& a, int bits) {
    if (a.zero()) return a;
    Big r;
    const int limbs = bits / 32, sh = bits % 32;
    r.d.assign(a.d.size() + limbs + 1, 0);
    for (size_t i = 0; i < a.d.size(); ++i) {
        uint64_t v = (uint64_t)a.d[i] << sh;
        r.d[i + limbs] |= (uint32_t)v;
        r.d[i + limbs + 1] |= (uint32_t)(v >> 32);
    }
    r.trim();
    return r;
}

int bitlen(const Big& a) {
    if (a.zero()) return 0;
    int b = 32 * (int)(a.d.size() - 1);
    uint32_t top = a.d.back();
    while (top) { ++b; top >>= 1; }
    return b;
}

Big fact(int n) {
    Big r(1);
    for (int i = 2; i <= n; ++i) r = mul(r, Big((uint64_t)i));
    return r;
}

// nearest double to sqrt(p/q), p > 0, q > 0, p/q < 2^100
double sqrt_ratio_rounded(const Big& p, const Big& q) {
    // k >= 0 with 2^104 q <= p 4^k < 2^106 q
    int k = std::max(0, (106 - (bitlen(p) - bitlen(q))) / 2);
    for (int it = 0; it < 8; ++it) {
        Big pk = shl(p, 2 * k);
        if (cmp(pk, shl(q, 104)) < 0) { ++k; continue; }
        if (cmp(pk, shl(q, 106)) >= 0) { --k; continue; }
        break;
    }
    const Big pk = shl(p, 2 * k);
    // largest M in [2^52, 2^53) with M^2 q <= p 4^k
    uint64_t lo = (uint64_t)1 << 52, hi = ((uint64_t)1 << 53) - 1;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo + 1) / 2;
        Big m(mid);
        if (cmp(mul(mul(m, m), q), pk) <= 0) lo = mid;
        else hi = mid - 1;
    }
    uint64_t M = lo;
    Big twoM1((uint64_t)2 * M + 1);
    if (cmp(shl(pk, 2), mul(mul(twoM1, twoM1), q)) > 0) ++M;
    return std::ldexp((double)M, -k);
}

double three_j_exact(int j1, int j2, int j3, int m1, int m2, int m3) {
    if (m1 + m2 + m3 != 0) return 0.0;
    if (j3 > j1 + j2 || j3 < std::abs(j1 - j2) || j1 < 0 || j2 < 0 || j3 < 0) return 0.0;
    if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
    const int tmin = std::max(0, std::max(j2 - j3 - m1, j1 - j3 + m2));
    const int tmax = std::min(j1 + j2 - j3, std::min(j1 - m1, j2 + m2));
    if (tmin > tmax) return 0.0;
    std::vector<Big> den;
    std::vector<int> sgn;
    for (int t = tmin; t <= tmax; ++t) {
        Big d = mul(mul(mul(fact(t), fact(j3 - j2 + t + m1)), mul(fact(j3 - j1 + t - m2), fact(j1 + j2 - j3 - t))),
                    mul(fact(j1 - t - m1), fact(j2 - t + m2)));
        den.push_back(d);
        sgn.push_back((t & 1) ? -1 : 1);
    }
    // S = sum sgn_t / den_t = (sum sgn_t prod_{t'!=t} den_t') / prod den_t
    Big DS(1), pos, neg;
    for (auto& d : den) DS = mul(DS, d);
    for (size_t i = 0; i < den.size(); ++i) {
        Big term(1);
        for (size_t j = 0; j < den.size(); ++j)
            if (j != i) term = mul(term, den[j]);
        if (sgn[i] > 0) pos = add(pos, term);
        else neg = add(neg, term);
    }
    int ssign;
    Big NS;
    const int c = cmp(pos, neg);
    if (c == 0) return 0.0;
    if (c > 0) { NS = sub(pos, neg); ssign = 1; }
    else { NS = sub(neg, pos); ssign = -1; }
    Big p = mul(mul(mul(fact(j1 + j2 - j3), fact(j1 - j2 + j3)), fact(-j1 + j2 + j3)),
                mul(mul(mul(fact(j1 + m1), fact(j1 - m1)), mul(fact(j2 + m2), fact(j2 - m2))),
                    mul(fact(j3 + m3), fact(j3 - m3))));
    p = mul(p, mul(NS, NS));
    Big q = mul(fact(j1 + j2 + j3 + 1), mul(DS, DS));
    const int phase = ((j1 - j2 - m3) % 2 + 2) % 2;
    const double v = sqrt_ratio_rounded(p, q);
    return (phase ? -1.0 : 1.0) * ssign * v;
}

}  // namespace

void threej_table_host(int jmax, double* t) {
    const int n = jmax + 1;
    for (int i = 0; i < n * n * 9; ++i) t[i] = 0.0;
    for (int jI = 0; jI <= jmax; ++jI)
        for (int jF = std::max(jI - 1, 0); jF <= std::min(jI + 1, jmax); ++jF)
            for (int kI = 0; kI <= jI; ++kI)
                for (int kF = std::max(kI - 1, 0); kF <= std::min(kI + 1, jF); ++kF)
                    t[jI + kI * n + (jF - jI + 1) * n * n + (kF - kI + 1) * n * n * 3] =
                        three_j_exact(jI, 1, jF, kI, kF - kI, -kF);
}

}  // namespace gain
