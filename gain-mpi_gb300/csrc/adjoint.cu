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

__global__ void k_adj_scale(int rows, int cols, const double* __restrict__ dLdS, const double* __restrict__ amp,
                            long ld_amp, double* __restrict__ G) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)rows * cols) return;
    const long r = i / cols, c = i - r * cols;
    G[i] = 2.0 * dLdS[i] * amp[r * ld_amp + c];
}

// C[m][n] = sum_k A[m][k] B[levels[k]][n]: 64 x 64 tiles, 16 x 16 threads, 4 x 4 outputs each.
constexpr int kTile = 64, kTk = 16;
__global__ void __launch_bounds__(256)
k_adj_gemm(int M, int N, int K, const double* __restrict__ A, long lda, const double* __restrict__ B, long ldb,
           const int* __restrict__ levels, double* __restrict__ C, long ldc) {
    __shared__ double sA[kTk][kTile + 1];
    __shared__ double sB[kTk][kTile + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kTk) {
        for (int t = threadIdx.x; t < kTile * kTk; t += 256) {
            const int mm = t / kTk, kk = t % kTk;           // A tile: 64 rows x 16 k
            const int gm = m0 + mm, gk = k0 + kk;
            sA[kk][mm] = (gm < M && gk < K) ? A[(long)gm * lda + gk] : 0.0;
            const int kb = t / kTile, nn = t % kTile;       // B tile: 16 k x 64 columns
            const int gk2 = k0 + kb, gn = n0 + nn;
            sB[kb][nn] = (gk2 < K && gn < N) ? B[(long)levels[gk2] * ldb + gn] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTk; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = sA[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = sB[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = __fma_rn(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
            if (gm < M && gn < N) C[(long)gm * ldc + gn] = acc[i][j];
        }
}

// One thread per (F, I) candidate: I across the block, F over the grid's y dimension; pairs
// outside the K-block window of F (|K_I - K_F| > 1) or with a vanishing factor return early.
__device__ void adj_dmu_one(const AdjArgs& a, int F, int I) {
    const int vF = a.vibF[F];
    if (vF < a.startF || vF >= a.endF) return;
    double w[3] = {0.0, 0.0, 0.0};
    int dsel = -1;   // component of the K-block form (one component per (F, I))
    if (a.wigner) {
        const long wi = 3 * ((long)a.levI[I] + (long)a.nlevelI *
                             ((long)a.levF[F] + (long)a.nlevelF * ((long)a.KI[I] + (long)a.maxdeg * a.KF[F])));
        w[0] = a.wigner[wi];
        w[1] = a.wigner[wi + 1];
        w[2] = a.wigner[wi + 2];
    } else {
        const int kI = a.KI[I], kF = a.KF[F];
        if (abs(kI - kF) > 1) return;
        const int tI = a.tauI[I], tF = a.tauF[F] & 1;
        const int eq = (kF == kI), neq = !eq, tneq = (tF != tI);
        const int c = (tF - tI) * eq + (tF - tI) * (kF - kI) * neq * tneq - neq * (!tneq);
        if (c == 0) return;
        const int n = a.jmax + 1;
        double m = a.threej[a.jI + kI * n + (a.jF - a.jI + 1) * n * n + (kF - kI + 1) * n * n * 3];
        if (kI != kF && kI * kF != 0) m *= kSqrt2Ref;
        m *= (double)c * parity_sign((kI % 3) * tI + kI) * parity_sign((kF % 3) * tF);
        dsel = 2 * eq + neq * (!tneq);
        w[dsel] = m;
    }
    double acc = 0.0;
    for (int b = 0; b < a.nb; ++b) acc = __fma_rn(a.dh[(long)b * a.ld_dh + F], a.vp[(long)b * a.ld_vp + I], acc);
    const long base = (long)(vF - a.startF) + (long)a.vibI[I] * a.ncontrF;
    const long ds = (long)a.dipN * a.ncontrF;
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (w[d] != 0.0) atomicAdd(&a.dmu[base + d * ds], w[d] * acc);
}

__global__ void __launch_bounds__(256)
k_adj_dmu(AdjArgs a) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= a.dimI) return;
    for (int F = blockIdx.y; F < a.dimF; F += gridDim.y) adj_dmu_one(a, F, I);
}

}  // namespace

cudaError_t launch_adj_scale(int rows, int cols, const double* dLdS, const double* amp, long ld_amp, double* G,
                             cudaStream_t st) {
    const long n = (long)rows * cols;
    if (n <= 0) return cudaSuccess;
    k_adj_scale<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rows, cols, dLdS, amp, ld_amp, G);
    return cudaGetLastError();
}

cudaError_t launch_adj_gemm(int M, int N, int K, const double* A, long lda, const double* B, long ldb,
                            const int* levels, double* C, long ldc, cudaStream_t st) {
    if (M <= 0 || N <= 0) return cudaSuccess;
    k_adj_gemm<<<dim3((N + kTile - 1) / kTile, (M + kTile - 1) / kTile), 256, 0, st>>>(M, N, K, A, lda, B, ldb,
                                                                                     levels, C, ldc);
    return cudaGetLastError();
}

cudaError_t launch_adj_dmu(const AdjArgs& a, cudaStream_t st) {
    if (a.dimF <= 0 || a.dimI <= 0 || a.nb <= 0) return cudaSuccess;
    k_adj_dmu<<<dim3((a.dimI + 255) / 256, a.dimF < 65535 ? a.dimF : 65535), 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace gain
