// Adjoint of the line-strength path: dL/dmu for a loss L over the line strengths of one
// block pair, given dL/dS.  With amp[b][u] = sum_Fs U[u][Fs] H[b][Fs], H = T_F^T h (the
// expansion's transpose), h[b][F] = sum_I M[F][I] v[b][I] and M[F][I] = factor(F, I) mu_d(F,I):
//   G[b][u]        = dL/dS[b][u] 2 amp[b][u]
//   dH[b][Fs]      = sum_u G[b][u] U[u][Fs]                         (FP64 GEMM)
//   dh[b][F]       = (T_F dH[b])[F]                                 (the expansion itself)
//   dM[F][I]       = sum_b dh[b][F] v[b][I]                         (only where M can be non-zero)
//   dL/dmu_d[vF][vI] += factor(F, I) dM[F][I] over the (F, I) with d(F, I) = d
// factor(F, I) is the K-block kernel's per-element factor (GPU/dipole_GPU.cu:457-509: 3j,
// the truncated 1/sqrt(2), the (tau, K) sign and component rules) or, in the
// rotational-symmetry form, the Wigner weights of all three components (:692-702).
#include "gain_internal.h"

namespace gain {
namespace {

__device__ __forceinline__ double parity_sign(int x) { return (x & 1) ? -1.0 : 1.0; }

template <class T>
__global__ void k_adj_scale(int rows, int cols, const double* __restrict__ dLdS, const double* __restrict__ amp,
                            long ld_amp, double two_scale, T* __restrict__ G) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)rows * cols) return;
    const long r = i / cols, c = i - r * cols;
    G[i] = (T)two_scale * (T)dLdS[i] * (T)amp[r * ld_amp + c];
}

// Register-tiled SIMT product: 64 x 64 output tiles, 16 x 16 threads, each thread the 4 x 4
// outputs (ty + 16 i, tx + 16 j), so a warp's shared-memory reads are broadcasts (rows) or 16
// consecutive words (columns).  Accumulation in T, one FMA per term in ascending inner order.
constexpr int kTile = 64, kTk = 16;

// C[m][n] = sum_k A[m][k] B[levels[k]][n]  (B is FP64 eigenvector storage, rounded to T)
template <class T>
__global__ void __launch_bounds__(256)
k_adj_gemm(int M, int N, int K, const T* __restrict__ A, long lda, const double* __restrict__ B, long ldb,
           const int* __restrict__ levels, T* __restrict__ C, long ldc) {
    __shared__ T sA[kTk][kTile + 1];
    __shared__ T sB[kTk][kTile];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
    T acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kTk) {
        for (int t = threadIdx.x; t < kTile * kTk; t += 256) {
            const int mm = t / kTk, kk = t % kTk;           // A tile: 64 rows x 16 k
            const int gm = m0 + mm, gk = k0 + kk;
            sA[kk][mm] = (gm < M && gk < K) ? A[(long)gm * lda + gk] : (T)0;
            const int kb = t / kTile, nn = t % kTile;       // B tile: 16 k x 64 columns
            const int gk2 = k0 + kb, gn = n0 + nn;
            sB[kb][nn] = (gk2 < K && gn < N) ? (T)B[(long)levels[gk2] * ldb + gn] : (T)0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTk; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = sA[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sB[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
            if (gm < M && gn < N) C[(long)gm * ldc + gn] = acc[i][j];
        }
}

// The half line strength's factor of (F, I) for the three dipole components: the K-block
// kernel's 3j, truncated 1/sqrt(2), sign and component rules (one component non-zero), or the
// rotational-symmetry form's Wigner weights.  Returns false when all three vanish or when F
// lies outside the dipole piece.
__device__ __forceinline__ bool adj_factor(const AdjArgs& a, int F, int I, double w[3]) {
    w[0] = w[1] = w[2] = 0.0;
    const int vF = a.vibF[F];
    if (vF < a.startF || vF >= a.endF) return false;
    if (a.wigner) {
        const long wi = 3 * ((long)a.levI[I] + (long)a.nlevelI *
                             ((long)a.levF[F] + (long)a.nlevelF * ((long)a.KI[I] + (long)a.maxdeg * a.KF[F])));
        w[0] = a.wigner[wi];
        w[1] = a.wigner[wi + 1];
        w[2] = a.wigner[wi + 2];
        return w[0] != 0.0 || w[1] != 0.0 || w[2] != 0.0;
    }
    const int kI = a.KI[I], kF = a.KF[F];
    if (abs(kI - kF) > 1) return false;
    const int tI = a.tauI[I], tF = a.tauF[F] & 1;
    const int eq = (kF == kI), neq = !eq, tneq = (tF != tI);
    const int c = (tF - tI) * eq + (tF - tI) * (kF - kI) * neq * tneq - neq * (!tneq);
    if (c == 0) return false;
    const int n = a.jmax + 1;
    double m = a.threej[a.jI + kI * n + (a.jF - a.jI + 1) * n * n + (kF - kI + 1) * n * n * 3];
    if (kI != kF && kI * kF != 0) m *= kSqrt2Ref;
    m *= (double)c * parity_sign((kI % 3) * tI + kI) * parity_sign((kF % 3) * tF);
    w[2 * eq + neq * (!tneq)] = m;
    return true;
}

// dM[F][I] = sum_b dh[b][F] vp[b][I] over one listed 64 x 64 (F, I) tile, then
// dL/dmu_d[vI][vF - startF] += factor_d(F, I) dM[F][I] (atomic: several (F, I) share an entry).
template <class T>
__global__ void __launch_bounds__(256)
k_adj_dm(AdjArgs a, const int2* __restrict__ tiles) {
    __shared__ T sH[kTk][kTile];
    __shared__ T sV[kTk][kTile];
    const int2 tile = tiles[blockIdx.x];
    const int f0 = tile.x, i0 = tile.y;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const T* dh = static_cast<const T*>(a.dh);
    const T* vp = static_cast<const T*>(a.vp);
    T acc[4][4] = {};
    for (int b0 = 0; b0 < a.nb; b0 += kTk) {
        for (int t = threadIdx.x; t < kTile * kTk; t += 256) {
            const int bb = t / kTile, c = t % kTile;        // both tiles: 16 states x 64 functions
            const int gb = b0 + bb;
            sH[bb][c] = (gb < a.nb && f0 + c < a.dimF) ? dh[(long)gb * a.ld_dh + f0 + c] : (T)0;
            sV[bb][c] = (gb < a.nb && i0 + c < a.dimI) ? vp[(long)gb * a.ld_vp + i0 + c] : (T)0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTk; ++kk) {
            T x[4], y[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) x[i] = sH[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) y[j] = sV[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(x[i], y[j], acc[i][j]);
        }
        __syncthreads();
    }
    T* dmu = static_cast<T*>(a.dmu);
    const long ds = (long)a.dipN * a.ncontrF;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int F = f0 + ty + 16 * i;
        if (F >= a.dimF) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int I = i0 + tx + 16 * j;
            double w[3];
            if (I >= a.dimI || !adj_factor(a, F, I, w)) continue;
            const long base = (long)(a.vibF[F] - a.startF) + (long)a.vibI[I] * a.ncontrF;
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if (w[d] != 0.0) atomicAdd(&dmu[base + d * ds], (T)w[d] * acc[i][j]);
        }
    }
}

// ---- the tensor-core form: operands of the two digit GEMMs, their refinement, the scatter
// out[p][b] = src[row(b) * ld + map[p]] for p < np, b < nb (0 where map[p] < 0 or b >= nb,
// up to the padded sizes np_pad x nb_pad; row(b) = rows[b], or b without rows).  32 x 32
// tiles through shared memory: the reads run along map (the source rows), the writes along b.
__global__ void __launch_bounds__(256)
k_gather_t(int np_pad, int nb, int nb_pad, const double* __restrict__ src, long ld, const int* __restrict__ rows,
           const int* __restrict__ map, double* __restrict__ out) {
    __shared__ double tile[32][33];
    const int p0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
    for (int i = ty; i < 32; i += 8) {
        const int b = b0 + i, p = p0 + tx;
        double v = 0.0;
        if (b < nb && p < np_pad) {
            const int c = map[p];
            if (c >= 0) v = src[(long)(rows ? rows[b] : b) * ld + c];
        }
        tile[i][tx] = v;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        const int p = p0 + i, b = b0 + tx;
        if (p < np_pad && b < nb_pad) out[(long)p * nb_pad + b] = tile[tx][i];
    }
}

// FP64 recomputation of the flagged entries of a digit product C[r][c] = sum_k A[r][k] B[c][k]
// (rows of length K, leading dimensions lda / ldb; one warp per entry).
__global__ void k_refine_rows(const int2* __restrict__ flags, const unsigned int* nflags, int max_flags,
                              const double* __restrict__ A, long lda, const double* __restrict__ B, long ldb, int K,
                              double* C, long ldc) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int n = min((int)*nflags, max_flags);
    for (int f = gw; f < n; f += nw) {
        const int2 rc = flags[f];
        const double* a = A + (long)rc.x * lda;
        const double* b = B + (long)rc.y * ldb;
        double acc = 0.0;
        for (int k = lane; k < K; k += 32) acc = __fma_rn(a[k], b[k], acc);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) C[(long)rc.x * ldc + rc.y] = acc;
    }
}

// dL/dmu_d[vI][vF - startF] += factor_d(F, I) dM[r][c] over the band of every F position r
// (columns [band_lo[r], band_hi[r]) of the lower positions; F = fmap[r], I = imap[c]).  One
// block per F position, its threads along the band.
__global__ void __launch_bounds__(256)
k_adj_scatter_band(AdjArgs a, const int* __restrict__ fmap, const int* __restrict__ imap,
                   const int* __restrict__ band_lo, const int* __restrict__ band_hi, const double* __restrict__ dM,
                   long ld) {
    const int r = blockIdx.x;
    const int F = fmap[r];
    if (F < 0) return;
    double* dmu = static_cast<double*>(a.dmu);
    const long ds = (long)a.dipN * a.ncontrF;
    for (int c = band_lo[r] + threadIdx.x; c < band_hi[r]; c += blockDim.x) {
        const int I = imap[c];
        double w[3];
        if (I < 0 || !adj_factor(a, F, I, w)) continue;
        const double v = dM[(long)r * ld + c];
        if (v == 0.0) continue;
        const long base = (long)(a.vibF[F] - a.startF) + (long)a.vibI[I] * a.ncontrF;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            if (w[d] != 0.0) atomicAdd(&dmu[base + d * ds], w[d] * v);
    }
}

}  // namespace

cudaError_t launch_gather_t(int np_pad, int nb, int nb_pad, const double* src, long ld, const int* rows,
                            const int* map, double* out, cudaStream_t st) {
    if (np_pad <= 0 || nb_pad <= 0) return cudaSuccess;
    const dim3 grid((np_pad + 31) / 32, (nb_pad + 31) / 32);
    k_gather_t<<<grid, 256, 0, st>>>(np_pad, nb, nb_pad, src, ld, rows, map, out);
    return cudaGetLastError();
}

cudaError_t launch_refine_rows(const int2* flags, const unsigned int* nflags, int max_flags, const double* A,
                               long lda, const double* B, long ldb, int K, double* C, long ldc, int max_blocks,
                               cudaStream_t st) {
    k_refine_rows<<<max_blocks, 256, 0, st>>>(flags, nflags, max_flags, A, lda, B, ldb, K, C, ldc);
    return cudaGetLastError();
}

cudaError_t launch_adj_scatter_band(const AdjArgs& a, int nrows, const int* fmap, const int* imap, const int* band_lo,
                                    const int* band_hi, const double* dM, long ld, cudaStream_t st) {
    if (nrows <= 0) return cudaSuccess;
    k_adj_scatter_band<<<nrows, 256, 0, st>>>(a, fmap, imap, band_lo, band_hi, dM, ld);
    return cudaGetLastError();
}

cudaError_t launch_adj_scale(int rows, int cols, const double* dLdS, const double* amp, long ld_amp,
                             double two_scale, void* G, bool fp32, cudaStream_t st) {
    const long n = (long)rows * cols;
    if (n <= 0) return cudaSuccess;
    const unsigned nblk = (unsigned)((n + 255) / 256);
    if (fp32)
        k_adj_scale<float><<<nblk, 256, 0, st>>>(rows, cols, dLdS, amp, ld_amp, two_scale, static_cast<float*>(G));
    else
        k_adj_scale<double><<<nblk, 256, 0, st>>>(rows, cols, dLdS, amp, ld_amp, two_scale, static_cast<double*>(G));
    return cudaGetLastError();
}

cudaError_t launch_adj_gemm(int M, int N, int K, const void* A, long lda, const double* B, long ldb,
                            const int* levels, void* C, long ldc, bool fp32, cudaStream_t st) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    const dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
    if (fp32)
        k_adj_gemm<float><<<grid, 256, 0, st>>>(M, N, K, static_cast<const float*>(A), lda, B, ldb, levels,
                                                static_cast<float*>(C), ldc);
    else
        k_adj_gemm<double><<<grid, 256, 0, st>>>(M, N, K, static_cast<const double*>(A), lda, B, ldb, levels,
                                                 static_cast<double*>(C), ldc);
    return cudaGetLastError();
}

int adj_tile() { return kTile; }

cudaError_t launch_adj_dm(const AdjArgs& a, const int* tiles, int ntiles, bool fp32, cudaStream_t st) {
    if (ntiles <= 0 || a.nb <= 0) return cudaSuccess;
    const int2* t = reinterpret_cast<const int2*>(tiles);
    if (fp32)
        k_adj_dm<float><<<ntiles, 256, 0, st>>>(a, t);
    else
        k_adj_dm<double><<<ntiles, 256, 0, st>>>(a, t);
    return cudaGetLastError();
}

}  // namespace gain
