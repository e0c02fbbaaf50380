// Line-list text on the device: every kept line of a block pair's last run formatted exactly
// as Output::OutputLinestrength prints it (BaseClasses/Output.cpp:99-111), compacted into one
// contiguous buffer in row-major (lower state, then upper state) order.
//
// Three launches over the rows x cols lines, 2048 lines per block (256 threads x 8 lines):
//   k_text_len    S/A/I of each line (line_eval), its text length (0 when not written) and
//                 the block's byte total;
//   k_text_offs   exclusive scan of the block totals (one block);
//   k_text_write  the block-local scan of the lengths, then each thread writes its lines.
// The length pass runs the same conversion as the write pass with a counting sink, so the
// offsets hold for any value (wide %f fields, three-digit exponents, NaN).
#include "gain_internal.h"
#include "linemath.cuh"
#include "linefmt.h"

namespace gain {
namespace {

constexpr int kTextThreads = 256, kTextItems = 8, kTextSpan = kTextThreads * kTextItems;

__device__ __forceinline__ long line_text(const TextArgs& t, long idx, fmt::Sink& s) {
    const int r = (int)(idx / t.cols), c = (int)(idx - (long)r * t.cols);
    const double a = t.amp[(long)r * t.ld + c];
    const LineVals v = line_eval(a, t.eI[r], t.eF[c], t.p);
    if (!v.keep) return 0;
    fmt::LineFields f;
    f.nu = v.nu;
    f.A = v.A;
    f.intensity = v.I;
    f.indexF = t.levF[c];
    f.jF = t.jF;
    f.gammaF = t.gammaF;
    f.indexI = t.levI[r];
    f.jI = t.jI;
    f.gammaI = t.gammaI;
    f.with_intensity = t.p.with_intensity;
    f.amps = t.with_amps ? &a : nullptr;
    f.namp = 1;
    const long n0 = s.n;
    fmt::put_line(s, f);
    return s.n - n0;
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
        fmt::Sink s{nullptr, 0, 0};
        const long n = line_text(t, idx, s);
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

// Exclusive scan of nblocks block totals in place; block_bytes[nblocks] = the text size.
__global__ void __launch_bounds__(kTextThreads) k_text_offs(unsigned long long* block_bytes, long nblocks) {
    unsigned long long carry = 0;
    for (long b0 = 0; b0 < nblocks; b0 += kTextThreads) {
        const long b = b0 + threadIdx.x;
        const unsigned long long v = b < nblocks ? block_bytes[b] : 0ull;
        unsigned long long all;
        const unsigned long long pre = block_exclusive_scan(v, &all);
        if (b < nblocks) block_bytes[b] = carry + pre;
        carry += all;
    }
    if (threadIdx.x == 0) block_bytes[nblocks] = carry;
}

__global__ void __launch_bounds__(kTextThreads) k_text_write(TextArgs t) {
    const long total = (long)t.rows * t.cols;
    const long base = (long)blockIdx.x * kTextSpan + (long)threadIdx.x * kTextItems;
    unsigned long long mine = 0;
    for (int i = 0; i < kTextItems; ++i)
        if (base + i < total) mine += t.lens[base + i];
    unsigned long long all;
    const unsigned long long pre = block_exclusive_scan(mine, &all);
    const unsigned long long off = t.block_bytes[blockIdx.x] + pre;   // bounded by the text size
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

cudaError_t launch_text_write(const TextArgs& t, cudaStream_t st) {
    const long nb = text_blocks((long)t.rows * t.cols);
    if (nb <= 0) return cudaSuccess;
    k_text_write<<<(unsigned)nb, kTextThreads, 0, st>>>(t);
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
