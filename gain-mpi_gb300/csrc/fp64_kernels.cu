// FP64 kernels of the line-strength path: the kernel-level drop-ins (K-block half line
// strength, vector expansion, dot product), the plain-path kernels (half line strength of
// the needed upper functions, transpose expansion, GEMV against resident upper vectors) and
// the S / A / I line assembly.
#include <algorithm>

#include "gain_internal.h"
#include "linemath.cuh"

namespace gain {
namespace {

__device__ __forceinline__ double parity_sign(int x) { return (x & 1) ? -1.0 : 1.0; }

// 3j table index of GpuManager.cpp:179 / dipole_GPU.cu:445
__device__ __forceinline__ int threej_index(int jI, int kI, int jF, int kF, int jmax) {
    const int n = jmax + 1;
    return jI + kI * n + (jF - jI + 1) * n * n + (kF - kI + 1) * n * n * 3;
}

// The rotational factor of one (lower, upper) primitive pair, as the reference kernel
// evaluates it (GPU/dipole_GPU.cu:490-495): dipole component and integer coefficient.
__device__ __forceinline__ void rot_factor(int kI, int kF, int tauI, int tauF, int* didx, int* c) {
    const int eq = (kF == kI), neq = !eq;
    const int tneq = (tauF != tauI);
    *didx = 2 * eq + neq * (!tneq);
    *c = (tauF - tauI) * eq + (tauF - tauI) * (kF - kI) * neq * tneq - neq * (!tneq);
}

// ---------------------------------------------------------------------------------------
// Drop-in K-block kernel.  One thread per upper primitive of the K block; lower functions
// of the three neighbouring K blocks are staged through shared memory 128 at a time.  Each
// output is accumulated in ascending lower index with one fused multiply-add per term, the
// same operation sequence as the reference kernel, so results agree bit for bit.
constexpr int kDropTile = 128;

__global__ void __launch_bounds__(kDropTile)
k_hls_kblock(int dimenF, int dimenI, int jI, int jF, int kF, const int* __restrict__ tauI,
             const int* __restrict__ tauF, const int* __restrict__ icorrI,
             const int* __restrict__ icorrF, int startF_idx, int startI_idx, int startFblock,
             int endFblock, int ncontrF, const int* __restrict__ kblock_size,
             const double* __restrict__ dipole_me, const double* __restrict__ vector,
             const double* __restrict__ threej, double* __restrict__ half_ls, int jmax,
             int dip_stride) {
    __shared__ double s_lsf[kDropTile];
    __shared__ double s_sgn[kDropTile];
    __shared__ int s_tau[kDropTile];
    __shared__ long s_off[kDropTile];

    const int f = blockIdx.x * kDropTile + threadIdx.x;
    const int irootF = startF_idx + f;
    const bool inF = f < dimenF;
    int icF = 0, tF = 0;
    if (inF) {
        icF = icorrF[irootF];
        tF = tauF[irootF] & 1;
    }
    const bool valid = inF && icF >= startFblock && icF < endFblock;
    icF -= startFblock;
    const long stride = (long)ncontrF * dip_stride;
    double acc = 0.0;
    int startI = startI_idx;
    for (int kI = max(kF - 1, 0); kI < kF + 2 && kI < jI + 1; ++kI) {
        const int kbs = kblock_size[kI];
        const double sq = (kI * kF != 0) ? kSqrt2Ref : 1.0;
        const double f3j = threej[threej_index(jI, kI, jF, kF, jmax)];
        int didx_same, c_same, didx_flip, c_flip;   // tau_I == tau_F and tau_I != tau_F cases
        rot_factor(kI, kF, tF, tF, &didx_same, &c_same);
        rot_factor(kI, kF, tF ^ 1, tF, &didx_flip, &c_flip);
        for (int base = 0; base < kbs; base += kDropTile) {
            const int loc = base + threadIdx.x;
            double lsf = 0.0, sg = 1.0;
            int ti = 0;
            long off = 0;
            if (loc < kbs) {
                const int ir = startI + loc;
                ti = tauI[ir];
                off = (long)icorrI[ir] * ncontrF;
                sg = parity_sign((kI % 3) * ti + kI);
                double ls = vector[ir];
                if (kF != kI) ls = __dmul_rn(ls, sq);
                lsf = __dmul_rn(ls, f3j);
            }
            __syncthreads();
            s_lsf[threadIdx.x] = lsf;
            s_sgn[threadIdx.x] = sg;
            s_tau[threadIdx.x] = ti;
            s_off[threadIdx.x] = off;
            __syncthreads();
            const int n = min(kDropTile, kbs - base);
            if (valid) {
                for (int i = 0; i < n; ++i) {
                    const double l = s_lsf[i];
                    if (l == 0.0) continue;
                    const int t = s_tau[i];
                    int didx, c;
                    if (t == tF) { didx = didx_same; c = c_same; }
                    else if (t == (tF ^ 1)) { didx = didx_flip; c = c_flip; }
                    else rot_factor(kI, kF, t, tF, &didx, &c);
                    const double ls = __dmul_rn(l, (double)c);
                    acc = __fma_rn(__dmul_rn(ls, s_sgn[i]), dipole_me[icF + s_off[i] + didx * stride], acc);
                }
            }
        }
        startI += kbs;
        if (startI >= dimenI) break;
    }
    if (valid) half_ls[irootF] = __dmul_rn(acc, parity_sign((kF % 3) * tF));
}

// ---------------------------------------------------------------------------------------
// device_expand_vectors (GPU/dipole_GPU.cu:859-889): one thread per primitive function.
__global__ void k_expand(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                         const int* __restrict__ ijterms, const int* __restrict__ icontr,
                         const int* __restrict__ N, const double* __restrict__ repres,
                         const double* __restrict__ vecI, double* __restrict__ vec) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= dimen) return;
    const int irow = icontr[r];
    const int ib = icontr[r + dimen];
    const int iterm = ijterms[irow + igamma * maxcoeff];
    const int nelem = N[irow];
    const long base = (long)ideg * Ntot + (long)ib * sdeg * Ntot;
    double acc = 0.0;
    for (int i = 0; i < nelem; ++i) acc = __fma_rn(vecI[iterm + i], repres[iterm + i + base], acc);
    vec[r] = acc;
}

// ---------------------------------------------------------------------------------------
// dot product with a device result: one CTA, strided partial sums, tree reduction.
__global__ void __launch_bounds__(1024) k_dot(int n, const double* __restrict__ x,
                                              const double* __restrict__ y, double* result) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc = __fma_rn(x[i], y[i], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) *result = acc;
    }
}

// ---------------------------------------------------------------------------------------
// Plain path: half line strength of the listed upper primitives.  Each CTA covers
// functions of one upper K; the lower functions come from the per-K support lists of the
// lower symmetry class, in ascending primitive order, so each output equals the
// reference kernel's value bit for bit (entries outside the support are zero and the
// reference skips them).
__global__ void __launch_bounds__(kHlsTile)
k_hls_needed(const HlsCta* __restrict__ ctas, const int* __restrict__ f_list, int jI, int jF,
             const int* __restrict__ tauI, const int* __restrict__ tauF,
             const int* __restrict__ icorrI, const int* __restrict__ icorrF,
             const int* __restrict__ sup_list, const int* __restrict__ sup_start,
             int startFblock, int endFblock, int ncontrF, const double* __restrict__ dipole_me,
             int dip_stride, const double* __restrict__ prim_vec, long ld_prim,
             const double* __restrict__ threej, int jmax, double* __restrict__ half_ls, long ld_h) {
    __shared__ double s_lsf[kHlsTile];
    __shared__ double s_sgn[kHlsTile];
    __shared__ int s_tau[kHlsTile];
    __shared__ long s_off[kHlsTile];
    // blockIdx.y: lower state of the batch
    prim_vec += (long)blockIdx.y * ld_prim;
    half_ls += (long)blockIdx.y * ld_h;
    const HlsCta cta = ctas[blockIdx.x];
    const int kF = cta.kF;
    const bool inF = (int)threadIdx.x < cta.f_count;
    int irootF = 0, icF = 0, tF = 0;
    if (inF) {
        irootF = f_list[cta.f_begin + threadIdx.x];
        icF = icorrF[irootF];
        tF = tauF[irootF] & 1;
    }
    const bool valid = inF && icF >= startFblock && icF < endFblock;
    icF -= startFblock;
    const long stride = (long)ncontrF * dip_stride;
    double acc = 0.0;
    for (int kI = max(kF - 1, 0); kI < kF + 2 && kI < jI + 1; ++kI) {
        const int s0 = sup_start[kI], ns = sup_start[kI + 1] - s0;
        const double sq = (kI * kF != 0) ? kSqrt2Ref : 1.0;
        const double f3j = threej[threej_index(jI, kI, jF, kF, jmax)];
        for (int base = 0; base < ns; base += kHlsTile) {
            const int loc = base + threadIdx.x;
            double lsf = 0.0, sg = 1.0;
            int ti = 0;
            long off = 0;
            if (loc < ns) {
                const int ir = sup_list[s0 + loc];
                ti = tauI[ir];
                off = (long)icorrI[ir] * ncontrF;
                sg = parity_sign((kI % 3) * ti + kI);
                double ls = prim_vec[ir];
                if (kF != kI) ls = __dmul_rn(ls, sq);
                lsf = __dmul_rn(ls, f3j);
            }
            __syncthreads();
            s_lsf[threadIdx.x] = lsf;
            s_sgn[threadIdx.x] = sg;
            s_tau[threadIdx.x] = ti;
            s_off[threadIdx.x] = off;
            __syncthreads();
            const int n = min(kHlsTile, ns - base);
            if (valid) {
                for (int i = 0; i < n; ++i) {
                    const double l = s_lsf[i];
                    if (l == 0.0) continue;
                    int didx, c;
                    rot_factor(kI, kF, s_tau[i], tF, &didx, &c);
                    const double ls = __dmul_rn(l, (double)c);
                    acc = __fma_rn(__dmul_rn(ls, s_sgn[i]), dipole_me[icF + s_off[i] + didx * stride], acc);
                }
            }
        }
    }
    if (valid) half_ls[irootF] = __dmul_rn(acc, parity_sign((kF % 3) * tF));
    else if (inF) half_ls[irootF] = 0.0;
}

__global__ void k_contract(int nsym, const int* __restrict__ rowptr, const int* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ h, long ld_h,
                           double* __restrict__ hsym, long ld_hs) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsym) return;
    h += (long)blockIdx.y * ld_h;
    hsym += (long)blockIdx.y * ld_hs;
    double acc = 0.0;
    for (int e = rowptr[s]; e < rowptr[s + 1]; ++e) acc = __fma_rn(h[col[e]], val[e], acc);
    hsym[s] = acc;
}

// expansion of a batch of stored vectors: blockIdx.y picks the level
// TV: storage of the vectors; TP: the arithmetic and output (double, or float for the FP32
// adjoint, where both operands are rounded to float before the product)
template <class TV, class TP>
__global__ void k_expand_levels(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                const int* __restrict__ ijterms, const int* __restrict__ icontr,
                                const int* __restrict__ N, const double* __restrict__ repres,
                                const TV* __restrict__ vecs, long ldv, const int* __restrict__ levels,
                                TP* __restrict__ prim, long ldp) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= dimen) return;
    const TV* vecI = vecs + (long)levels[blockIdx.y] * ldv;
    const int irow = icontr[r];
    const int ib = icontr[r + dimen];
    const int iterm = ijterms[irow + igamma * maxcoeff];
    const int nelem = N[irow];
    const long base = (long)ideg * Ntot + (long)ib * sdeg * Ntot;
    TP acc = 0;
    for (int i = 0; i < nelem; ++i) acc = fma((TP)vecI[iterm + i], (TP)repres[iterm + i + base], acc);
    prim[(long)blockIdx.y * ldp + r] = acc;
}

// One warp per upper state: its vector is read once and dotted with the half line
// strengths of up to kGemvBatch lower states (each dot: lane-strided FMA, tree reduction).
constexpr int kGemvBatch = 8;
__global__ void __launch_bounds__(256)
k_gemv_batch(int nrows, int n, const double* __restrict__ U, long ldu, const int* __restrict__ levels,
             const double* __restrict__ x, long ldx, int nb, double* __restrict__ out, long ldo) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nrows) return;
    const double* row = U + (long)levels[warp] * ldu;
    double acc[kGemvBatch];
#pragma unroll
    for (int g = 0; g < kGemvBatch; ++g) acc[g] = 0.0;
    for (int i = lane; i < n; i += 32) {
        const double u = __ldg(row + i);
#pragma unroll
        for (int g = 0; g < kGemvBatch; ++g)
            if (g < nb) acc[g] = __fma_rn(u, __ldg(x + (long)g * ldx + i), acc[g]);
    }
#pragma unroll
    for (int g = 0; g < kGemvBatch; ++g) {
        double a = acc[g];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0 && g < nb) out[(long)g * ldo + warp] = a;
    }
}

__global__ void k_scatter_select(int dimen, const int* __restrict__ sym_of,
                                 const double* __restrict__ coef, const double* __restrict__ vec,
                                 double* __restrict__ prim) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= dimen) return;
    const int s = sym_of[r];
    prim[r] = s >= 0 ? __dmul_rn(vec[s], coef[r]) : 0.0;
}

// Row error of H_sym = H_prim T (T the upper expansion) from that of H_prim: with sigma a
// bound of ||T||_2 and gam that of the FP64 contraction's rounding (relative to |T||H|),
//   ||err_sym||_2 <= sigma ||err_prim||_2 + gam sigma ||H_prim row||_2.
// rowerr2 is a squared norm in units of 2^{2 e[row]}; one block per row, rounded up.
__global__ void __launch_bounds__(256)
k_contract_rowerr(int rows, const double* __restrict__ Hp, long ldp, int ncols, float* __restrict__ rowerr2,
                  const int* __restrict__ e, double sigma, double gam) {
    __shared__ double red[8];
    const int r = blockIdx.x;
    if (r >= rows) return;
    double ss = 0.0;
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
        const double h = Hp[(long)r * ldp + c];
        ss = __fma_ru(h, h, ss);
    }
    for (int o = 16; o > 0; o >>= 1) ss = __dadd_ru(ss, __shfl_xor_sync(0xffffffffu, ss, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = __dadd_ru(t, red[w]);
        const double hn = __dmul_ru(__dsqrt_ru(t), ldexp(1.0, -e[r]));
        const double v = __fma_ru(__dmul_ru(gam, sigma), hn, __dmul_ru(sigma, __dsqrt_ru((double)rowerr2[r])));
        rowerr2[r] = __double2float_ru(__dmul_ru(__dmul_ru(v, v), 1.0000001));
    }
}

__global__ void k_add(double* __restrict__ acc, const double* __restrict__ x, long n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        acc[i] += x[i];
}

// S / A / I of every amplitude (non-degenerate symmetries), Output.cpp:52-112.
// Grid-stride over the rows x cols lines (each pass coalesced); the kept-line count is
// reduced in the block and added once per block.
__global__ void __launch_bounds__(256)
k_lines(int rows, int cols, const double* __restrict__ amp, long ld,
        const double* __restrict__ eI, const double* __restrict__ eF, LineParams p,
        double* __restrict__ S, double* __restrict__ A, double* __restrict__ I,
        unsigned char* __restrict__ keep, unsigned long long* nkeep) {
    __shared__ unsigned int warp_kept[8];
    const long total = (long)rows * cols;
    unsigned int kept = 0;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / cols), c = (int)(idx - (long)r * cols);
        const LineVals v = line_eval(amp, (long)r * ld + c, eI[r], eF[c], p);
        kept += v.keep;
        if (S) S[idx] = v.ls;
        if (A) A[idx] = v.A;
        if (I) I[idx] = v.I;
        if (keep) keep[idx] = (unsigned char)v.keep;
    }
    for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
    if ((threadIdx.x & 31) == 0) warp_kept[threadIdx.x >> 5] = kept;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < 8; ++w) t += warp_kept[w];
        if (t) atomicAdd(nkeep, t);
    }
}

// Lines whose Einstein A may lie on either side of THRESH_LINE given the amplitudes'
// certified bounds (Output.cpp:95 keeps a line when A >= THRESH_LINE): the line strength is
// evaluated, in the reference's operation order, at |amp| - bound and at |amp| + bound for
// every amplitude it combines; S and then A are monotone in each |amp| under round to
// nearest, so the true A lies between the two results.  A line with A_lo < THRESH_LINE <=
// A_hi is listed for recomputation in FP64.
__global__ void __launch_bounds__(256)
k_thresh_flag(int rows, int cols, const double* __restrict__ amp, long ld, const float* __restrict__ bnd, long ldb,
              const double* __restrict__ eI, const double* __restrict__ eF, LineParams p, int2* list,
              unsigned int* count, int cap) {
    const long total = (long)rows * cols;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const int r = (int)(idx / cols), c = (int)(idx - (long)r * cols);
        const double nu = eF[c] - eI[r];
        if (!(nu >= p.freq_lo && nu <= p.freq_hi && nu >= 1e-40)) continue;   // not written in any case
        double lo, hi;
        if (p.nslot == 0) {
            const double a = fabs(amp[(long)r * ld + c]), b = (double)bnd[(long)r * ldb + c];
            if (b == 0.0) continue;
            const double al = a > b ? a - b : 0.0, ah = a + b;
            lo = __dmul_rn(al, al);
            hi = __dmul_rn(ah, ah);
        } else {
            lo = 0.0;
            hi = 0.0;
            bool any = false;
            for (int s = 0; s < p.nslot; ++s) {
                const long o = (long)p.slot[s] * p.slot_stride + (long)r * ld + c;
                const double a = fabs(amp[o]), b = (double)bnd[(long)p.slot[s] * p.slot_stride + (long)r * ldb + c];
                any = any || b != 0.0;
                const double al = a > b ? a - b : 0.0, ah = a + b;
                lo = __dadd_rn(lo, __dmul_rn(al, al));
                hi = __dadd_rn(hi, __dmul_rn(ah, ah));
            }
            if (!any) continue;
            lo = __ddiv_rn(lo, (double)p.ndegI);
            hi = __ddiv_rn(hi, (double)p.ndegI);
            if (p.reduced_deg) {
                lo = __dmul_rn(lo, (double)p.ndegI);
                hi = __dmul_rn(hi, (double)p.ndegI);
            }
        }
        const double anu = fabs(nu);
        const double Alo = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(p.acoef_2jI1, lo), anu), anu), anu);
        const double Ahi = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(p.acoef_2jI1, hi), anu), anu), anu);
        if (Alo < p.thresh && Ahi >= p.thresh) {
            const unsigned int k = atomicAdd(count, 1u);
            if ((int)k < cap) list[k] = make_int2(r, c);
        }
    }
}

// dst[pairs[2i]] = src[pairs[2i+1]], and the bound of that entry (when given) becomes 0
__global__ void k_patch(int n, const long long* __restrict__ pairs, const double* __restrict__ src, double* dst,
                        float* dstbnd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long d = pairs[2 * i], s = pairs[2 * i + 1];
    dst[d] = src[s];
    if (dstbnd) dstbnd[d] = 0.0f;
}

}  // namespace

cudaError_t launch_thresh_flag(int rows, int cols, const double* amp, long ld, const float* bnd, long ldb,
                               const double* eI, const double* eF, const LineParams& p, int2* list,
                               unsigned int* count, int cap, cudaStream_t st) {
    const long total = (long)rows * cols;
    if (total <= 0) return cudaSuccess;
    const long blocks = std::min<long>((total + 255) / 256, 152L * 8);
    k_thresh_flag<<<(unsigned)blocks, 256, 0, st>>>(rows, cols, amp, ld, bnd, ldb, eI, eF, p, list, count, cap);
    return cudaGetLastError();
}

cudaError_t launch_patch(int n, const long long* pairs, const double* src, double* dst, float* dstbnd,
                         cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_patch<<<(n + 255) / 256, 256, 0, st>>>(n, pairs, src, dst, dstbnd);
    return cudaGetLastError();
}

cudaError_t launch_hls_kblock(int dimenF, int dimenI, int jI, int jF, int kF, const int* tauI,
                              const int* tauF, const int* icorrI, const int* icorrF, int startF_idx,
                              int startI_idx, int startFblock, int endFblock, int ncontrF,
                              const int* kblock_size, const double* dipole_me,
                              const double* vector, const double* threej, double* half_ls,
                              int jmax, int dip_stride, cudaStream_t st) {
    if (dimenF <= 0) return cudaSuccess;
    k_hls_kblock<<<(dimenF + kDropTile - 1) / kDropTile, kDropTile, 0, st>>>(
        dimenF, dimenI, jI, jF, kF, tauI, tauF, icorrI, icorrF, startF_idx, startI_idx,
        startFblock, endFblock, ncontrF, kblock_size, dipole_me, vector, threej, half_ls, jmax,
        dip_stride);
    return cudaGetLastError();
}

cudaError_t launch_expand(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                          const int* ijterms, const int* icontr, const int* N,
                          const double* repres, const double* vecI, double* vec, cudaStream_t st) {
    if (dimen <= 0) return cudaSuccess;
    k_expand<<<(dimen + 255) / 256, 256, 0, st>>>(dimen, igamma, maxcoeff, ideg, sdeg, Ntot,
                                                   ijterms, icontr, N, repres, vecI, vec);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Rotational-symmetry (Euler) half line strength, the drop-in for
// device_compute_1st_half_ls_flipped_dipole_shared_rotsym_nontrove (GPU/dipole_GPU.cu:641-723):
// one thread per upper primitive F in the dipole block, summing over every lower primitive
// I in ascending order; per I the three components enter as fma(w0, mu0, w1 mu1), then
// fma(w2, mu2, .), accumulated with one fused multiply-add -- the reference's own order,
// so the values are bit-identical.  In this form K holds the degeneracy index and ktau the
// rotational level index of each primitive.
constexpr int kRotTile = 128;

__global__ void __launch_bounds__(kRotTile)
k_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int maxdeg, const int* __restrict__ kI,
             const int* __restrict__ kF, const int* __restrict__ ktauI, const int* __restrict__ ktauF,
             const int* __restrict__ icorrI, const int* __restrict__ icorrF, int startFblock, int endFblock,
             int ncontrF, const double* __restrict__ dipole_me, long dstride, const double* __restrict__ wigner,
             const double* __restrict__ vector, double* __restrict__ half_ls) {
    __shared__ double s_v[kRotTile];
    __shared__ long s_ic[kRotTile];
    __shared__ int s_lv[kRotTile], s_dg[kRotTile];
    const int t = threadIdx.x;
    const int f = blockIdx.x * kRotTile + t;
    bool valid = f < dimenF;
    long icF = 0, wF = 0;
    if (valid) {
        const int c = icorrF[f];
        valid = c >= startFblock && c < endFblock;
        icF = c - startFblock;
        wF = (long)ktauF[f] * nlevelI * 3 + (long)kF[f] * maxdeg * nlevelI * nlevelF * 3;
    }
    const long wdeg = (long)nlevelI * nlevelF * 3;
    double acc = 0.0;
    for (int b = 0; b < dimenI; b += kRotTile) {
        const int i = b + t;
        if (i < dimenI) {
            s_ic[t] = (long)icorrI[i] * ncontrF;
            s_lv[t] = ktauI[i];
            s_dg[t] = kI[i];
            s_v[t] = vector[i];
        }
        __syncthreads();
        const int n = min(kRotTile, dimenI - b);
        if (valid) {
            for (int j = 0; j < n; ++j) {
                const long d = icF + s_ic[j];
                const double mu0 = dipole_me[d], mu1 = dipole_me[d + dstride], mu2 = dipole_me[d + 2 * dstride];
                const long w = (long)s_lv[j] * 3 + wF + (long)s_dg[j] * wdeg;
                const double tt = __fma_rn(wigner[w + 2], mu2, __fma_rn(wigner[w], mu0, __dmul_rn(wigner[w + 1], mu1)));
                acc = __fma_rn(s_v[j], tt, acc);
            }
        }
        __syncthreads();
    }
    if (valid) half_ls[f] = acc;
}

cudaError_t launch_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int maxdeg, const int* kI,
                              const int* kF, const int* ktauI, const int* ktauF, const int* icorrI, const int* icorrF,
                              int startFblock, int endFblock, int ncontrF, const double* dipole_me, int dip_stride,
                              const double* wigner, const double* vector, double* half_ls, cudaStream_t st) {
    if (dimenF <= 0) return cudaSuccess;
    k_hls_rotsym<<<(dimenF + kRotTile - 1) / kRotTile, kRotTile, 0, st>>>(
        dimenF, dimenI, nlevelI, nlevelF, maxdeg, kI, kF, ktauI, ktauF, icorrI, icorrF, startFblock, endFblock,
        ncontrF, dipole_me, (long)ncontrF * dip_stride, wigner, vector, half_ls);
    return cudaGetLastError();
}

cudaError_t launch_dot(int n, const double* x, const double* y, double* result, cudaStream_t st) {
    k_dot<<<1, 1024, 0, st>>>(n, x, y, result);
    return cudaGetLastError();
}

cudaError_t launch_hls_needed(const HlsCta* ctas, int ncta, const int* f_list, int jI, int jF,
                              const int* tauI, const int* tauF, const int* icorrI,
                              const int* icorrF, const int* sup_list, const int* sup_start,
                              int startFblock, int endFblock, int ncontrF,
                              const double* dipole_me, int dip_stride, const double* prim_vec,
                              long ld_prim, const double* threej, int jmax, double* half_ls,
                              long ld_h, int nbatch, cudaStream_t st) {
    if (ncta <= 0 || nbatch <= 0) return cudaSuccess;
    k_hls_needed<<<dim3(ncta, nbatch), kHlsTile, 0, st>>>(
        ctas, f_list, jI, jF, tauI, tauF, icorrI, icorrF, sup_list, sup_start, startFblock, endFblock,
        ncontrF, dipole_me, dip_stride, prim_vec, ld_prim, threej, jmax, half_ls, ld_h);
    return cudaGetLastError();
}

cudaError_t launch_contract(int nsym, const int* rowptr, const int* col, const double* val,
                            const double* h, long ld_h, double* hsym, long ld_hs, int nbatch,
                            cudaStream_t st) {
    if (nsym <= 0 || nbatch <= 0) return cudaSuccess;
    k_contract<<<dim3((nsym + 255) / 256, nbatch), 256, 0, st>>>(nsym, rowptr, col, val, h, ld_h, hsym, ld_hs);
    return cudaGetLastError();
}

template <class TV, class TP>
static cudaError_t expand_levels_t(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                   const int* ijterms, const int* icontr, const int* N, const double* repres,
                                   const TV* vecs, long ldv, const int* levels, TP* prim, long ldp, int nbatch,
                                   cudaStream_t st) {
    if (dimen <= 0 || nbatch <= 0) return cudaSuccess;
    k_expand_levels<TV, TP><<<dim3((dimen + 255) / 256, nbatch), 256, 0, st>>>(
        dimen, igamma, maxcoeff, ideg, sdeg, Ntot, ijterms, icontr, N, repres, vecs, ldv, levels, prim, ldp);
    return cudaGetLastError();
}

cudaError_t launch_expand_levels(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                 const int* ijterms, const int* icontr, const int* N, const double* repres,
                                 const double* vecs, long ldv, const int* levels, double* prim, long ldp,
                                 int nbatch, cudaStream_t st) {
    return expand_levels_t(dimen, igamma, maxcoeff, ideg, sdeg, Ntot, ijterms, icontr, N, repres, vecs, ldv, levels,
                           prim, ldp, nbatch, st);
}

cudaError_t launch_expand_levels(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                 const int* ijterms, const int* icontr, const int* N, const double* repres,
                                 const double* vecs, long ldv, const int* levels, float* prim, long ldp,
                                 int nbatch, cudaStream_t st) {
    return expand_levels_t(dimen, igamma, maxcoeff, ideg, sdeg, Ntot, ijterms, icontr, N, repres, vecs, ldv, levels,
                           prim, ldp, nbatch, st);
}

cudaError_t launch_expand_levels(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                 const int* ijterms, const int* icontr, const int* N, const double* repres,
                                 const float* vecs, long ldv, const int* levels, float* prim, long ldp,
                                 int nbatch, cudaStream_t st) {
    return expand_levels_t(dimen, igamma, maxcoeff, ideg, sdeg, Ntot, ijterms, icontr, N, repres, vecs, ldv, levels,
                           prim, ldp, nbatch, st);
}

cudaError_t launch_gemv_batch(int nrows, int n, const double* U, long ldu, const int* levels, const double* x,
                              long ldx, int nbatch, double* out, long ldo, cudaStream_t st) {
    if (nrows <= 0 || nbatch <= 0) return cudaSuccess;
    if (nbatch > kGemvBatch) return cudaErrorInvalidValue;
    k_gemv_batch<<<(nrows + 7) / 8, 256, 0, st>>>(nrows, n, U, ldu, levels, x, ldx, nbatch, out, ldo);
    return cudaGetLastError();
}

cudaError_t launch_scatter_select(int dimen, const int* sym_of, const double* coef,
                                  const double* vec, double* prim, cudaStream_t st) {
    if (dimen <= 0) return cudaSuccess;
    k_scatter_select<<<(dimen + 255) / 256, 256, 0, st>>>(dimen, sym_of, coef, vec, prim);
    return cudaGetLastError();
}

cudaError_t launch_contract_rowerr(int rows, const double* Hp, long ldp, int ncols, float* rowerr2, const int* e,
                                  double sigma, double gam, cudaStream_t st) {
    if (rows <= 0) return cudaSuccess;
    k_contract_rowerr<<<rows, 256, 0, st>>>(rows, Hp, ldp, ncols, rowerr2, e, sigma, gam);
    return cudaGetLastError();
}

cudaError_t launch_add(double* acc, const double* x, long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const long blocks = std::min<long>((n + 255) / 256, 4096);
    k_add<<<(unsigned)blocks, 256, 0, st>>>(acc, x, n);
    return cudaGetLastError();
}

cudaError_t launch_lines(int rows, int cols, const double* amp, long ld, const double* eI,
                         const double* eF, LineParams p, double* S, double* A, double* I,
                         unsigned char* keep, unsigned long long* nkeep, cudaStream_t st) {
    const long total = (long)rows * cols;
    if (total <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long blocks = (total + 255) / 256;
    const long cap = (long)(sms > 0 ? sms : 152) * 4;   // one wave at four resident blocks per SM
    if (blocks > cap) blocks = cap;
    k_lines<<<(unsigned)blocks, 256, 0, st>>>(rows, cols, amp, ld, eI, eF, p, S, A, I, keep, nkeep);
    return cudaGetLastError();
}

}  // namespace gain
