// Line-list text on the device: every kept line of a block pair's last run formatted exactly
// as Output::OutputLinestrength prints it (BaseClasses/Output.cpp:99-111), compacted into one
// contiguous buffer in row-major (lower state, then upper state) order.
//
// Three launches over the rows x cols lines, 1024 lines per block (256 threads x 4 lines):
//   k_text_len    S/A/I of each line (line_eval), its text length (0 when not written) and
//                 the block's byte total; the lengths come from the value ranges where those
//                 fix them and from the conversion itself elsewhere (wide %f fields,
//                 three-digit exponents), so they equal what the write pass writes;
//   k_text_offs   exclusive scan of the block totals, the total and the largest block;
//   k_text_write  the block-local scan of the lengths; each thread formats its lines into
//                 shared memory, placed at the block's output offset modulo 16, and the block
//                 copies its text out in aligned 16-byte stores (whole L2 sectors, no partial
//                 writes).  A block whose text does not fit shared memory writes directly.
#include <atomic>

#include "gain_internal.h"
#include "linemath.cuh"
#include "linefmt.h"

namespace gain {
namespace {

constexpr int kTextThreads = 256, kTextItems = 4, kTextSpan = kTextThreads * kTextItems;
constexpr int kStageMax = 200 * 1024;   // shared-memory staging of one block's text

// Could the printed intensity (%16.9E: ten significant digits) of a line whose device value
// is I differ from what the host C library's exp gives?  Both exp results lie within 1 ulp of
// the exact value, so the two intensities differ by a relative
//   delta <= 2^-52 (7 + 2 e2 / (1 - e2)),  e2 = exp(-beta nu)
// (the rounding of 1 - e2 amplifies the exp difference); five times that is allowed.  The
// line is hard when a ten-digit rounding boundary lies within delta of I (or the decimal
// exponent could change, or I is zero, tiny, huge or not finite).  x = |I| 10^(9 - e) comes
// from the correctly rounded power of ten (pow10[k + 300] = 10^k) and one rounded product: a
// relative error of at most 2^-52, covered by the margin.  The decimal exponent e starts from
// the binary one and is corrected by comparing x with 10^9 and 10^10 (exact doubles).
__device__ __forceinline__ bool intensity_hard(double I, double e2, const double* __restrict__ pow10) {
    const double a = fabs(I);
    if (!(a >= 1e-290 && a <= 1e290)) return true;
    if (!(e2 < 1.0)) return true;
    const double delta = 0x1p-52 * (40.0 + 8.0 * e2 / (1.0 - e2));
    if (!(delta < 1e-6)) return true;
    const int e2b = (int)((__double_as_longlong(a) >> 52) & 0x7ff) - 1023;   // a is normal here
    int k = 9 - (int)floorf((float)e2b * 0.30103f);
    k = max(-300, min(300, k));
    double x = a * __ldg(&pow10[k + 300]);
    if (x < 1e9 && k < 300) x = a * __ldg(&pow10[k + 301]);
    else if (x >= 1e10 && k > -300) x = a * __ldg(&pow10[k + 299]);
    if (!(x >= 1e9 + 1.0 && x <= 1e10 - 2.0)) return true;
    const double fr = x - floor(x);
    return fabs(fr - 0.5) <= (delta + 0x1p-50) * x + 1e-6;
}

// Intensity the host gave for line idx (binary search of the override list), or v_dev.
__device__ __forceinline__ double intensity_of(const TextArgs& t, long idx, double v_dev) {
    int lo = 0, hi = t.n_ovr;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (t.ovr_idx[mid] < idx) lo = mid + 1;
        else hi = mid;
    }
    return lo < t.n_ovr && t.ovr_idx[lo] == idx ? t.ovr_val[lo] : v_dev;
}

// The fields of line idx; false when the line is not written.  a_out receives the printed
// amplitudes (kMaxDegSlots at most); eI_out / e2_out (optional) the lower energy and the
// exp(-beta nu) of the intensity.
__device__ __forceinline__ bool line_fields(const TextArgs& t, long idx, double* a_out, fmt::LineFields& f,
                                            double* eI_out = nullptr, double* e2_out = nullptr) {
    const int r = (int)(idx / t.cols), c = (int)(idx - (long)r * t.cols);
    const long off = (long)r * t.ld + c;
    const LineVals v = line_eval(t.amp, off, t.eI[r], t.eF[c], t.p);
    if (!v.keep) return false;
    if (eI_out) *eI_out = t.eI[r];
    if (e2_out) *e2_out = v.e2;
    int namp = 1;
    if (t.p.nslot == 0) {
        a_out[0] = t.amp[off];
    } else {
        namp = t.p.nslot;
        for (int s = 0; s < namp; ++s) a_out[s] = t.amp[off + (long)t.p.slot[s] * t.p.slot_stride];
    }
    f.nu = v.nu;
    f.A = v.A;
    f.intensity = (t.p.with_intensity && t.n_ovr > 0) ? intensity_of(t, idx, v.I) : v.I;
    f.indexF = t.levF[c];
    f.jF = t.jF;
    f.gammaF = t.gammaF;
    f.indexI = t.levI[r];
    f.jI = t.jI;
    f.gammaI = t.gammaI;
    f.with_intensity = t.p.with_intensity;
    f.amps = t.with_amps ? a_out : nullptr;
    f.namp = namp;
    return true;
}

__device__ __forceinline__ long line_text(const TextArgs& t, long idx, fmt::Sink& s) {
    double a[kMaxDegSlots];
    fmt::LineFields f;
    if (!line_fields(t, idx, a, f)) return 0;
    const long n0 = s.n;
    fmt::put_line(s, f);
    return s.n - n0;
}

__device__ __forceinline__ long line_length(const TextArgs& t, long idx) {
    double a[kMaxDegSlots];
    fmt::LineFields f;
    double eI = 0.0, e2 = 0.0;
    if (!line_fields(t, idx, a, f, &eI, &e2)) return 0;
    if (t.hard && t.p.with_intensity && intensity_hard(f.intensity, e2, t.pow10)) {
        const unsigned int k = atomicAdd(t.nhard, 1u);
        if ((int)k < t.hard_cap) t.hard[k] = TextArgs::HardLine{(long long)idx, f.A, f.nu, eI, f.intensity};
    }
    return fmt::line_len(f);
}

// Block-wide exclusive scan of one value per thread (256 threads); returns the prefix and
// sets *total.
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long* total) {
    __shared__ unsigned long long warp_sum[kTextThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    unsigned long long before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kTextThreads / 32; ++w) {
        const unsigned long long s = warp_sum[w];
        if (w < warp) before += s;
        all += s;
    }
    __syncthreads();
    *total = all;
    return before + x - v;
}

__global__ void __launch_bounds__(kTextThreads) k_text_len(TextArgs t) {
    const long total = (long)t.rows * t.cols;
    const long base = (long)blockIdx.x * kTextSpan + (long)threadIdx.x * kTextItems;
    unsigned long long sum = 0, kept = 0;
    for (int i = 0; i < kTextItems; ++i) {
        const long idx = base + i;
        if (idx >= total) break;
        const long n = line_length(t, idx);
        t.lens[idx] = (uint32_t)n;
        sum += (unsigned long long)n;
        kept += n > 0;
    }
    unsigned long long all, nk;
    block_exclusive_scan(sum, &all);
    block_exclusive_scan(kept, &nk);
    if (threadIdx.x == 0) {
        t.block_bytes[blockIdx.x] = all;
        if (nk) atomicAdd(t.nkeep, nk);
    }
}

// Exclusive scan of nblocks block totals in place; block_bytes[nblocks] = the text size,
// block_bytes[nblocks + 2] = the largest block total.
__global__ void __launch_bounds__(kTextThreads) k_text_offs(unsigned long long* block_bytes, long nblocks) {
    unsigned long long carry = 0, mx = 0;
    for (long b0 = 0; b0 < nblocks; b0 += kTextThreads) {
        const long b = b0 + threadIdx.x;
        const unsigned long long v = b < nblocks ? block_bytes[b] : 0ull;
        mx = v > mx ? v : mx;
        unsigned long long all;
        const unsigned long long pre = block_exclusive_scan(v, &all);
        if (b < nblocks) block_bytes[b] = carry + pre;
        carry += all;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = y > mx ? y : mx;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(&block_bytes[nblocks + 2], mx);
    if (threadIdx.x == 0) block_bytes[nblocks] = carry;
}

// The staged write: dynamic shared memory of at least the largest block's text + 16 bytes.
__global__ void __launch_bounds__(kTextThreads) k_text_write_staged(TextArgs t, long block0) {
    extern __shared__ __align__(16) char stage[];
    const long blk = block0 + blockIdx.x;
    const long total = (long)t.rows * t.cols;
    const long base = blk * kTextSpan + (long)threadIdx.x * kTextItems;
    unsigned long long mine = 0;
    for (int i = 0; i < kTextItems; ++i)
        if (base + i < total) mine += t.lens[base + i];
    unsigned long long all;
    const unsigned long long pre = block_exclusive_scan(mine, &all);
    const unsigned long long D = t.block_bytes[blk];
    const int pad = (int)(D & 15u);
    fmt::Sink s{stage + pad + pre, 0, (long)(all - pre)};
    for (int i = 0; i < kTextItems; ++i) {
        const long idx = base + i;
        if (idx >= total) break;
        if (t.lens[idx]) line_text(t, idx, s);
    }
    __syncthreads();
    // stage[pad + j] -> text[D + j], j < all, both 16-byte aligned from j = head on
    const unsigned long long lim = t.text_size > D ? t.text_size - D : 0ull;
    const long n = (long)(all < lim ? all : lim);
    char* dst = t.text + D;
    const long h0 = (16 - pad) & 15;
    const long head = h0 < n ? h0 : n;
    for (long j = threadIdx.x; j < head; j += kTextThreads) dst[j] = stage[pad + j];
    const long nbody = (n - head) / 16;
    const uint4* src4 = reinterpret_cast<const uint4*>(stage + pad + head);
    uint4* dst4 = reinterpret_cast<uint4*>(dst + head);
    for (long j = threadIdx.x; j < nbody; j += kTextThreads) dst4[j] = src4[j];
    for (long j = head + nbody * 16 + threadIdx.x; j < n; j += kTextThreads) dst[j] = stage[pad + j];
}

__global__ void __launch_bounds__(kTextThreads) k_text_write(TextArgs t, long block0) {
    const long blk = block0 + blockIdx.x;
    const long total = (long)t.rows * t.cols;
    const long base = blk * kTextSpan + (long)threadIdx.x * kTextItems;
    unsigned long long mine = 0;
    for (int i = 0; i < kTextItems; ++i)
        if (base + i < total) mine += t.lens[base + i];
    unsigned long long all;
    const unsigned long long pre = block_exclusive_scan(mine, &all);
    const unsigned long long off = t.block_bytes[blk] + pre;   // bounded by the text size
    fmt::Sink s{t.text + off, 0, (long)(t.text_size > off ? t.text_size - off : 0)};
    for (int i = 0; i < kTextItems; ++i) {
        const long idx = base + i;
        if (idx >= total) break;
        if (t.lens[idx]) line_text(t, idx, s);
    }
}

// One conversion per value: out[i * stride ...] holds the text of vals[i], lens[i] its length.
__global__ void k_format_values(long n, const double* __restrict__ vals, int conv, int width, int prec,
                                char* __restrict__ out, int stride, int* __restrict__ lens) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fmt::Sink c{nullptr, 0, 0};
    if (conv == 'E') fmt::put_E(c, vals[i], width, prec); else fmt::put_F(c, vals[i], width, prec);
    lens[i] = (int)c.n;
    if (c.n > stride) return;
    fmt::Sink s{out + i * (long)stride, 0, stride};
    if (conv == 'E') fmt::put_E(s, vals[i], width, prec); else fmt::put_F(s, vals[i], width, prec);
}

}  // namespace

long text_blocks(long lines) { return (lines + kTextSpan - 1) / kTextSpan; }

cudaError_t launch_text_len(const TextArgs& t, cudaStream_t st) {
    const long nb = text_blocks((long)t.rows * t.cols);
    if (nb <= 0) return cudaSuccess;
    k_text_len<<<(unsigned)nb, kTextThreads, 0, st>>>(t);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_text_offs<<<1, kTextThreads, 0, st>>>(t.block_bytes, nb);
    return cudaGetLastError();
}

cudaError_t launch_text_write(const TextArgs& t, unsigned long long max_block_bytes, long b0, long b1,
                              cudaStream_t st) {
    const long nb = text_blocks((long)t.rows * t.cols);
    if (b1 > nb) b1 = nb;
    if (b0 < 0 || b1 <= b0) return cudaSuccess;
    if (max_block_bytes + 16 <= (unsigned long long)kStageMax) {
        static std::atomic<unsigned long long> done{0};   // bit per device ordinal (< 64)
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (!(done.load() & (1ull << (dev & 63)))) {
            e = cudaFuncSetAttribute(k_text_write_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, kStageMax);
            if (e != cudaSuccess) return e;
            done.fetch_or(1ull << (dev & 63));
        }
        const size_t smem = (size_t)((max_block_bytes + 16 + 15) & ~15ull);
        k_text_write_staged<<<(unsigned)(b1 - b0), kTextThreads, smem, st>>>(t, b0);
    } else {
        k_text_write<<<(unsigned)(b1 - b0), kTextThreads, 0, st>>>(t, b0);
    }
    return cudaGetLastError();
}

cudaError_t launch_format_values(long n, const double* vals, int conv, int width, int prec, char* out, int stride,
                                 int* lens, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_format_values<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, vals, conv, width, prec, out, stride, lens);
    return cudaGetLastError();
}

}  // namespace gain

extern "C" {

int gain_format_line_native(char* buf, size_t cap, double nu, int indexF, int jF, int gammaF, int indexI, int jI,
                            int gammaI, double A, int with_intensity, double intensity, const double* amps,
                            int namp) {
    if (!buf || cap == 0) return 0;
    gain::fmt::LineFields f;
    f.nu = nu;
    f.A = A;
    f.intensity = intensity;
    f.indexF = indexF;
    f.jF = jF;
    f.gammaF = gammaF;
    f.indexI = indexI;
    f.jI = jI;
    f.gammaI = gammaI;
    f.with_intensity = with_intensity;
    f.amps = amps;
    f.namp = namp;
    gain::fmt::Sink c{nullptr, 0, 0};
    gain::fmt::put_line(c, f);
    if ((size_t)c.n >= cap) return -(int)c.n;
    gain::fmt::Sink s{buf, 0, (long)cap - 1};
    gain::fmt::put_line(s, f);
    buf[s.n] = 0;
    return (int)s.n;
}

long gain_line_length_native(double nu, int indexF, int jF, int gammaF, int indexI, int jI, int gammaI, double A,
                             int with_intensity, double intensity, const double* amps, int namp) {
    gain::fmt::LineFields f;
    f.nu = nu;
    f.A = A;
    f.intensity = intensity;
    f.indexF = indexF;
    f.jF = jF;
    f.gammaF = gammaF;
    f.indexI = indexI;
    f.jI = jI;
    f.gammaI = gammaI;
    f.with_intensity = with_intensity;
    f.amps = amps;
    f.namp = namp;
    return gain::fmt::line_len(f);
}

int gain_format_value(char* buf, size_t cap, double x, int conv, int width, int prec) {
    if (!buf || cap == 0 || (conv != 'E' && conv != 'f') || prec < 0 || prec > (conv == 'E' ? 17 : 9)) return 0;
    gain::fmt::Sink c{nullptr, 0, 0};
    if (conv == 'E') gain::fmt::put_E(c, x, width, prec); else gain::fmt::put_F(c, x, width, prec);
    if ((size_t)c.n >= cap) return -(int)c.n;
    gain::fmt::Sink s{buf, 0, (long)cap - 1};
    if (conv == 'E') gain::fmt::put_E(s, x, width, prec); else gain::fmt::put_F(s, x, width, prec);
    buf[s.n] = 0;
    return (int)s.n;
}

}  // extern "C"
