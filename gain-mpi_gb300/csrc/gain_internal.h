// Internal declarations shared by the translation units of libgainls.so.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include "../../include/gain_ls.h"

namespace gain {

// ---------------------------------------------------------------- error reporting
gain_status set_error(gain_status s, const char* fmt, ...);
void clear_error();
gain_status cuda_fail(cudaError_t e, const char* what);

#define GAIN_CUDA(call)                                                   \
    do {                                                                  \
        cudaError_t e__ = (call);                                         \
        if (e__ != cudaSuccess) return ::gain::cuda_fail(e__, #call);     \
    } while (0)

#define GAIN_TRY(call)                                                    \
    do {                                                                  \
        gain_status s__ = (call);                                         \
        if (s__ != GAIN_OK) return s__;                                   \
    } while (0)

// the reference's truncated 1/sqrt(2), GPU/dipole_GPU.cu:24
constexpr double kSqrt2Ref = 0.70710678118;

// exact Wigner 3j table (threej.cpp)
void threej_table_host(int jmax, double* table);

// ---------------------------------------------------------------- FP64 kernels (fp64_kernels.cu)
cudaError_t launch_hls_kblock(int dimenF, int dimenI, int jI, int jF, int kF, const int* tauI,
                              const int* tauF, const int* icorrI, const int* icorrF, int startF_idx,
                              int startI_idx, int startFblock, int endFblock, int ncontrF,
                              const int* kblock_size, const double* dipole_me,
                              const double* vector, const double* threej, double* half_ls,
                              int jmax, int dip_stride, cudaStream_t st);
cudaError_t launch_expand(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                          const int* ijterms, const int* icontr, const int* N,
                          const double* repres, const double* vecI, double* vec, cudaStream_t st);
cudaError_t launch_dot(int n, const double* x, const double* y, double* result, cudaStream_t st);
// ---------------------------------------------------------------- adjoint (adjoint.cu)
struct AdjArgs {
    int dimF, dimI, nb;                        // primitive dimensions, lower states
    const int *vibF, *vibI, *KF, *KI, *tauF, *tauI, *levF, *levI;
    int jI, jF, jmax;
    const double* threej;
    const double* wigner;                      // non-null: rotational-symmetry form
    int nlevelI, nlevelF, maxdeg;
    int startF, endF, ncontrF, dipN;
    // arrays of the chain's precision (double, or float with fp32)
    const void* dh;                            // [nb][ld_dh] dL/dh, primitive upper index
    long ld_dh;
    const void* vp;                            // [nb][ld_vp] lower vectors, primitive index
    long ld_vp;
    void* dmu;                                 // [3][dipN][ncontrF] accumulated
};
// G = two_scale dL/dS amp in double or float
cudaError_t launch_adj_scale(int rows, int cols, const double* dLdS, const double* amp, long ld_amp,
                             double two_scale, void* G, bool fp32, cudaStream_t st);
// C = A U[levels]: A and C double or float, the FP64 eigenvectors rounded to the chain's precision
cudaError_t launch_adj_gemm(int M, int N, int K, const void* A, long lda, const double* B, long ldb,
                            const int* levels, void* C, long ldc, bool fp32, cudaStream_t st);
// functions per side of one (F, I) tile of launch_adj_dm
int adj_tile();
// dL/dmu over the listed (F, I) tiles: tiles = ntiles pairs (first F, first I)
cudaError_t launch_adj_dm(const AdjArgs& a, const int* tiles, int ntiles, bool fp32, cudaStream_t st);
// out[p][b] = src[(rows ? rows[b] : b) * ld + map[p]] (0 where map[p] < 0 or b >= nb), the
// [np_pad][nb_pad] transpose-gather that lays out a digit GEMM operand
cudaError_t launch_gather_t(int np_pad, int nb, int nb_pad, const double* src, long ld, const int* rows,
                            const int* map, double* out, cudaStream_t st);
// FP64 recomputation of flagged C[r][c] = sum_k A[r][k] B[c][k]
cudaError_t launch_refine_rows(const int2* flags, const unsigned int* nflags, int max_flags, const double* A,
                               long lda, const double* B, long ldb, int K, double* C, long ldc, int max_blocks,
                               cudaStream_t st);
// dL/dmu (double) from the band entries dM[r][c], c in [band_lo[r], band_hi[r]) of nrows F positions
cudaError_t launch_adj_scatter_band(const AdjArgs& a, int nrows, const int* fmap, const int* imap, const int* band_lo,
                                    const int* band_hi, const double* dM, long ld, cudaStream_t st);

cudaError_t launch_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int maxdeg, const int* kI,
                              const int* kF, const int* ktauI, const int* ktauF, const int* icorrI, const int* icorrF,
                              int startFblock, int endFblock, int ncontrF, const double* dipole_me, int dip_stride,
                              const double* wigner, const double* vector, double* half_ls, cudaStream_t st);

// Plain FP64 path: one CTA table entry covers up to kHlsTile upper functions of one K block.
struct HlsCta {
    int kF;        // upper K of every function in this CTA
    int f_begin;   // offset into the needed-F list
    int f_count;   // <= kHlsTile
    int pad;
};
constexpr int kHlsTile = 128;

// half_ls restricted to the needed upper primitives (F list), summing over the lower
// support lists per K block. Writes half_ls[F] (primitive index) for every listed F.
cudaError_t launch_hls_needed(const HlsCta* ctas, int ncta, const int* f_list, int jI, int jF,
                              const int* tauI, const int* tauF, const int* icorrI,
                              const int* icorrF, const int* sup_list, const int* sup_start,
                              int startFblock, int endFblock, int ncontrF,
                              const double* dipole_me, int dip_stride, const double* prim_vec,
                              long ld_prim, const double* threej, int jmax, double* half_ls,
                              long ld_h, int nbatch, cudaStream_t st);

// hsym[s] = sum_{e in row s} h[col[e]] * val[e]  (transpose of the expansion), per batch row
cudaError_t launch_contract(int nsym, const int* rowptr, const int* col, const double* val,
                            const double* h, long ld_h, double* hsym, long ld_hs, int nbatch,
                            cudaStream_t st);

// expansion of the stored vectors vecs[levels[b]] into prim[b] (b < nbatch)
cudaError_t launch_expand_levels(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                 const int* ijterms, const int* icontr, const int* N, const double* repres,
                                 const double* vecs, long ldv, const int* levels, double* prim, long ldp,
                                 int nbatch, cudaStream_t st);
// the same in FP32 arithmetic (the FP32 adjoint): vectors of either precision, float output
cudaError_t launch_expand_levels(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                 const int* ijterms, const int* icontr, const int* N, const double* repres,
                                 const double* vecs, long ldv, const int* levels, float* prim, long ldp,
                                 int nbatch, cudaStream_t st);
cudaError_t launch_expand_levels(int dimen, int igamma, int maxcoeff, int ideg, int sdeg, int Ntot,
                                 const int* ijterms, const int* icontr, const int* N, const double* repres,
                                 const float* vecs, long ldv, const int* levels, float* prim, long ldp,
                                 int nbatch, cudaStream_t st);

// out[b*ldo + u] = sum_f U[level[u]*ldu + f] * x[b*ldx + f], u < nrows, b < nbatch <= 8
constexpr int kPlainBatch = 8;
cudaError_t launch_gemv_batch(int nrows, int n, const double* U, long ldu, const int* levels, const double* x,
                              long ldx, int nbatch, double* out, long ldo, cudaStream_t st);

// gather-expand of a selection expansion: prim[r] = coef[r] * vec[sym_of[r]] (sym_of<0 -> 0)
cudaError_t launch_scatter_select(int dimen, const int* sym_of, const double* coef,
                                  const double* vec, double* prim, cudaStream_t st);

// row error bound of H_prim T from that of H_prim (split path with a mixing expansion)
cudaError_t launch_contract_rowerr(int rows, const double* Hp, long ldp, int ncols, float* rowerr2, const int* e,
                                  double sigma, double gam, cudaStream_t st);
// acc[i] += x[i], i < n
cudaError_t launch_add(double* acc, const double* x, long n, cudaStream_t st);

// S, A, I of a [rows x cols] amplitude block, Output.cpp:52-112
constexpr int kMaxDegSlots = 9;   // degenerate component pairs of one line (maxdeg <= 3)
struct LineParams {
    double acoef_2jI1;   // ACOEF * (2 jI + 1), the first product of Output.cpp:93
    double cmcoef, gnsF, two_jF1;
    double beta, zpe, q_part, thresh, freq_lo, freq_hi;
    int with_intensity;
    // Degenerate states (Output.cpp:78-91): nslot > 0 sums amp^2 over the listed component
    // slots (idegF outer, idegI inner, those passing DegeneracyFilter), divides by ndegI and,
    // with reduced_deg (SYMMETRY REDUCED and both states degenerate), multiplies by ndegI.
    // nslot = 0: one amplitude per line, S = amp^2.
    int nslot, ndegI, reduced_deg;
    long slot_stride;              // doubles from one slot to the next
    int slot[kMaxDegSlots];
};
cudaError_t launch_lines(int rows, int cols, const double* amp, long ld, const double* eI,
                         const double* eF, LineParams p, double* S, double* A, double* I,
                         unsigned char* keep, unsigned long long* nkeep, cudaStream_t st);
// lines whose A lies within its certified bound of THRESH_LINE -> list (at most cap, count all)
cudaError_t launch_thresh_flag(int rows, int cols, const double* amp, long ld, const float* bnd, long ldb,
                               const double* eI, const double* eF, const LineParams& p, int2* list,
                               unsigned int* count, int cap, cudaStream_t st);
// dst[pairs[2i]] = src[pairs[2i+1]] for i < n; dstbnd (optional) zeroed at the same offsets
cudaError_t launch_patch(int n, const long long* pairs, const double* src, double* dst, float* dstbnd,
                         cudaStream_t st);

// ---------------------------------------------------------------- line-list text (linetext.cu)
struct TextArgs {
    int rows, cols;
    const double* amp;
    long ld;
    const double *eI, *eF;
    LineParams p;
    const int *levI, *levF;                // printed level indices (0-based) of rows / columns
    int jI, jF, gammaI, gammaF, with_amps;
    uint32_t* lens;                        // [rows*cols] text length of each line (0: not written)
    unsigned long long* block_bytes;       // [text_blocks + 3]: block offsets, the total, -, the largest block
    unsigned long long* nkeep;             // lines written
    char* text;
    unsigned long long text_size;          // bytes of text (the write pass stays inside)
    // Intensity column: lines whose printed intensity could differ from the host C library's
    // (the device exp and the host exp may differ in the last bits) are listed by the length
    // pass; the host evaluates their intensity with its own exp and both passes then print
    // those values (ovr_idx sorted, n_ovr entries)
    struct HardLine { long long idx; double A, nu, eI, I; };
    HardLine* hard;                        // may be null (no collection)
    const double* pow10;                   // [601]: pow10[k + 300] = 10^k correctly rounded
    unsigned int* nhard;
    int hard_cap;
    const long long* ovr_idx;
    const double* ovr_val;
    int n_ovr;
};
long text_blocks(long lines);
cudaError_t launch_text_len(const TextArgs& t, cudaStream_t st);     // lens, offsets, total, nkeep
// the text itself; max_block_bytes = the largest block total (block_bytes[text_blocks + 2])
// blocks [b0, b1) of the text
cudaError_t launch_text_write(const TextArgs& t, unsigned long long max_block_bytes, long b0, long b1,
                              cudaStream_t st);
cudaError_t launch_format_values(long n, const double* vals, int conv, int width, int prec, char* out,
                                 int stride, int* lens, cudaStream_t st);

}  // namespace gain
