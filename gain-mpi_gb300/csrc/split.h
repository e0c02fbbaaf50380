// Split-precision (Ozaki-style) tensor-core path: internal interface.
//
// Every FP64 operand row x is written as x = 2^e (sum_{i<s} d_i 2^{-(i+1) beta} + r),
// |r| <= 2^{-s beta - 1}, with balanced integer digits d_i (|d_0| <= 2^beta,
// |d_i| <= 2^{beta-1}) stored as BF16 (exact for beta <= 8).  A product of two rows is
// sum over digit pairs (i, j), i + j < s, of an integer dot product computed exactly by
// BF16 tcgen05 MMAs with FP32 accumulation (exact while every partial sum is an integer
// below 2^24, certified per output by Cauchy-Schwarz on per-row digit norms), weighted
// by 2^{-(i+j) beta} and summed in double-float in tensor memory.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace gain {
namespace split {

constexpr int BM = 128;     // output rows per tile (TMEM lanes)
constexpr int BN = 128;     // output columns per tile
constexpr int BK = 64;      // inner elements per stage (one 128-byte swizzle row of BF16)
constexpr int KSTEP = 2;    // k-blocks per pipeline stage (one barrier wait per 8 MMAs)
constexpr int STAGES = 3;   // stages of KSTEP k-blocks (64 KB each)
constexpr int MAX_CHUNKS = 8;
constexpr int MAX_SLICES = 10;

struct Tile {
    int m0, n0;     // first output row (A row) / column (B row)
    int a_k0;       // A inner coordinate of k-block 0
    int b_k0;       // B inner coordinate of k-block 0
    int nkb;        // k-blocks of BK
    int group;      // grouped launch: the tile's group; -1 in any launch: an empty slot of the schedule
    int pad[2];
};

struct Prod {
    int ia, ib;     // digit index of A and of B
    int t;          // ia + ib (weight 2^{-t beta})
    int chunk;      // inner-dimension chunk
    // Products of one weight and chunk may share an accumulator (a fused group): open = the
    // first of its group (the accumulator starts from zero), close = the last (the epilogue
    // drains it).  Unfused products have both.
    int open, close;
    int pad[2];
};

// Fixed-point position of the exact recombination: the running sum of the digit products
// of one output is an int64 in units of 2^{-kFixTotal} of 2^{eA+eB}, i.e. 2^{-fix_bits(beta)}
// of the digit-product units 2^{-2 beta}.
constexpr int kFixTotal = 50;
__host__ __device__ constexpr int fix_bits(int beta) { return kFixTotal - 2 * beta; }

// Per-row data of a sliced operand (x^ = x 2^{-e}; all norms rounded up).
struct RowStats {
    int* e;          // scale exponent (row values < 2^e)
    int* nnz;        // non-zero count
    float* l2;       // ||x^||_2
    float* dn;       // [rows * nchunks]: max_i ||d_i restricted to chunk||_2 (exactness certificate)
    float* dnv;      // [rows * MAX_SLICES]: ||d_i||_2 over the whole row
    float* rnv;      // [rows * MAX_SLICES]: ||x^ - X^(n)||_2, X^(n) = sum_{i<=n} d_i 2^{-(i+1) beta}
    float* inerr;    // optional: ||input error of the row||_2 in units of 2^e
};

struct GemmGroup;

struct GemmArgs {
    const Tile* tiles;
    int ntiles;
    // grouped launch: per-group arguments and tensor maps (device memory); tiles, ntiles and
    // err are the launch's, every other field comes from the tile's group
    const GemmGroup* groups;
    const Prod* prods;
    int nprods;
    int nchunks;
    int beta;
    int slices;
    double* out;
    long ldo;
    RowStats A, B;
    // bound of the fixed-point recombination (units of 2^{eA+eB}): nprods 2^{-kFixTotal}
    float c_fix;
    // worst-case rounding bound of an FP64 dot product of the same two rows, per unit of
    // ||x^||_2 ||y^||_2: (K + 64) 2^-53; a line is certified when its bound is within
    // max(tol |value|, that FP64 bound)
    float c_f64;
    // GEMM1: per row, sum over columns of (bound in units of 2^{eA})^2 (atomic add), may be null
    float* rowerr2;
    // optional: largest |value| over valid outputs (atomic max on the IEEE bits)
    unsigned long long* absmax;
    // flags
    int flag_mode;          // 0: inexact accumulation only; 1: also bound > tol |value|
    float tol;
    int2* flags;
    unsigned int* nflags;
    int max_flags;
    int rows_valid, cols_valid;
    int* err;               // device error word (0 ok, else timeout code)
    // optional: the absolute error bound of every output (float, rounded up; +inf where the
    // exact-accumulation certificate failed), bnd[row * ldb + col]
    float* bnd;
    long ldb;
    // largest number of products a fused group adds into one accumulator (0 or 1: none); the
    // exactness certificate then bounds that many products' sum
    int fuse;
};

// One group of a grouped launch: a block pair's operands (tensor maps) and arguments.
struct alignas(64) GemmGroup {
    CUtensorMap tmA, tmB;
    GemmArgs args;
};

size_t gemm_smem_bytes();
// The kernels' attributes on the current device (done by the first launch otherwise; call it
// before capturing launches into a graph).
cudaError_t prepare_device();
// pair: CTA pairs computing 256 x 128 tiles (tile m0 multiples of 256, rows padded to 256;
// the B operand's map with 64-row boxes)
cudaError_t launch_gemm(const CUtensorMap& tmA, const CUtensorMap& tmB, const GemmArgs& a,
                        int num_sms, cudaStream_t st, bool pair);

// Tensor map of a digit array [slices][rows_pad][kpad] BF16 (box 64 x box_rows x 1, 128B
// swizzle; box_rows 128, or 64 for the B operand of a CTA pair).
bool make_digit_map(CUtensorMap* map, void* base, int kpad, int rows_pad, int slices, int box_rows = BM);

// One persistent launch over the tiles of several groups (block pairs): a.tiles holds
// ntiles = units x k entries, unit u taking entries u, u + units, ... (empty slots have
// group -1); a.groups the groups; max_slices / max_chunks bound every group's.
cudaError_t launch_gemm_grouped(const GemmArgs& a, int units, int max_slices, int max_chunks, cudaStream_t st,
                                bool pair);

struct SliceArgs {
    const double* src;      // source rows
    long ld_src;
    const int* src_rows;    // optional source row per output row
    int nrows;              // output rows to produce
    int ncols;              // source columns
    const int* col_map;     // optional destination column per source column
    const int* col_inv;     // optional source column per destination column (-1: padding);
                            // with it (or with no map at all) the four-column kernel runs
    int kpad;               // destination row length
    long slice_stride;      // rows_pad * kpad
    __nv_bfloat16* digits;
    int slices, beta;
    int nchunks;            // chunks of the destination inner dimension for dn
    // source-column range of each chunk (the column map is increasing): chunk c covers the
    // sources mapped into destination k-blocks [c n/nch, (c+1) n/nch) of the GEMM
    int src_chunk[MAX_CHUNKS + 1];
    RowStats st;
    const float* inerr2_prev;  // optional: squared row error in units of 2^{2 e_prev}
    const int* e_prev;         // exponent those units refer to
    int grid_limit;            // CTAs at most (0: one per row)
};
cudaError_t launch_slice(const SliceArgs& a, cudaStream_t st);
// Several slicings in one launch: args[g] (device memory) produces the rows
// offs[g] <= r < offs[g + 1] of the flat row range [0, rows); all use the same kernel.
struct SliceGroups {
    const SliceArgs* args;
    const int* offs;
    int n, rows;
};
// The kernel a slicing runs on: S for the four-column kernel of S slices, 0 for the general one.
int slice_kernel_of(const SliceArgs& a);
cudaError_t launch_slice_grouped(const SliceGroups& g, int kernel, cudaStream_t st);

// Rotational-dipole band matrix of one block pair (rows: padded upper functions,
// columns: W band positions starting at band_k0[row] of the padded lower layout).
struct BandArgs {
    int fpad, W;
    const int* f_prim;      // primitive index of each padded upper row (-1: padding)
    const double* f_coef;
    const int* band_k0;
    int kpadI;
    const int* i_prim;      // primitive index of each padded lower column (-1: padding)
    const double* i_coef;
    const int *KI, *tauI, *vibI, *KF, *tauF, *vibF;
    int jI, jF, jmax;
    const double* threej;
    const double* dipole;
    int dipN, startF, endF, ncontrF;
    double* band;
    // rotational-symmetry form (GPU/dipole_GPU.cu:641-723) when non-null: dense in K, the entry
    // of (F, I) is sum_d wigner[d + 3 (tauI + nlevelI (tauF + nlevelF (KI + maxdeg KF)))] mu_d,
    // with tau = level index and K = degeneracy index
    const double* wigner;
    int nlevelI, nlevelF, maxdeg;
    // symmetric functions that combine primitives of one K: when f_ptr is non-null, upper row
    // r is sum_q f_val[q] prim f_col[q] over q in [f_ptr[r], f_ptr[r+1]) and lower column c
    // likewise through i_ptr / i_col / i_val; the entry is the double sum of the primitive
    // entries (f_prim / f_coef / i_prim / i_coef are then unused)
    const int *f_ptr, *f_col, *i_ptr, *i_col;
    const double *f_val, *i_val;
};
cudaError_t launch_band(const BandArgs& a, cudaStream_t st);
// one bounded mbarrier wait on a barrier nothing arrives on (err gets code 9 when it gives up)
cudaError_t launch_wait_selftest(unsigned long long limit_ns, int* err, cudaStream_t st);

// FP64 recomputation of flagged first-GEMM outputs (H entries).
struct RefineHArgs {
    const int2* flags;
    const unsigned int* nflags;
    int max_flags;
    const double* vecs;     // lower eigenvectors [levels][nsize]
    int nsize;
    const int* row_level;   // level of each batch row
    const int* i_sym;       // symmetry index of each padded lower column (-1: padding)
    const int* band_k0;
    const int* band_len;    // per padded upper row
    const double* band;
    int W;
    double* H;
    long ldh;
    const int* eA;
    float* rowerr2;
};
cudaError_t launch_refine_h(const RefineHArgs& a, int max_blocks, cudaStream_t st);

// FP64 recomputation of flagged amplitudes.
struct RefineAmpArgs {
    const int2* flags;
    const unsigned int* nflags;
    int max_flags;
    const double* U;        // upper eigenvectors [levels][nsize]
    int nsize;
    const int* col_level;   // level of each output column
    const int* colpos;      // padded position of each upper symmetry index
    const double* H;
    long ldh;
    const float* h_inerr;   // ||first-GEMM error of the H row||_2 in units of 2^{eH}
    const int* eH;
    double* amp;
    long lda;
    float* bnd;             // optional: the recomputed amplitude's error bound, bnd[r * ldb + c]
    long ldb;
    double tol;
    const unsigned long long* absmax;    // largest |amp| of the run (IEEE bits)
    double amp_floor;                    // sqrt(s_floor): certification domain |amp| >= floor*max
    unsigned long long* uncertified;     // in the domain
    unsigned long long* uncertified_weak;  // below it
};
cudaError_t launch_refine_amp(const RefineAmpArgs& a, int max_blocks, cudaStream_t st);

}  // namespace split
}  // namespace gain
