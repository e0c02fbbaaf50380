/* gain_ls.h -- C ABI of the GB300 line-strength library (libgainls.so).
 *
 * Drop-in replacement for GAIN-MPI's GPU line-strength path: the kernel wrappers of
 * GPU/dipole_GPU.h and the device work GpuManager (BaseClasses/GpuManager.h) orchestrates.
 * Plain pointers and sizes only; every entry point returns a gain_status and never aborts
 * the process (the reference calls MPI_Abort through LogErrorAndAbort on any CUDA error,
 * BaseClasses/GpuManager.cpp:80-93, common/BaseProcess.cpp:42-52).
 *
 * Two layers:
 *   1. kernel-level entry points with the reference wrappers' arguments and semantics
 *      (device pointers, asynchronous on the caller's stream);
 *   2. an engine that owns device memory (basis sets, expansion tables, dipole,
 *      eigenvectors) and computes whole (J'',Gamma'') -> (J',Gamma') block pairs, through
 *      either the reference's plain FP64 method or the split-precision tensor-core method.
 */
#ifndef GAIN_LS_H
#define GAIN_LS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GAIN_ABI_VERSION 1

typedef enum gain_status {
    GAIN_OK = 0,
    GAIN_ERR_INVALID_ARG = 1,   /* rejected on the host before any launch */
    GAIN_ERR_OOM = 2,           /* device or pinned allocation failed */
    GAIN_ERR_CUDA = 3,          /* a CUDA runtime / driver call failed */
    GAIN_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up */
    GAIN_ERR_TOL_NOT_MET = 5,   /* split path: some lines could not be certified */
    GAIN_ERR_NOT_READY = 6,     /* a required upload has not happened */
    GAIN_ERR_UNSUPPORTED = 7    /* valid input outside what this build implements */
} gain_status;

/* Message describing the most recent failure on the calling thread ("" if none). */
const char* gain_last_error_string(void);
const char* gain_status_string(gain_status s);
int gain_abi_version(void);

/* ======================= layer 1: kernel-level drop-ins ============================ */

/* One upper K-block kF of the half line strength.
 * Replaces compute_gpu_half_linestrength_ (GPU/dipole_GPU.h:23-26, GPU/dipole_GPU.cu:185-210)
 * with the same arguments in the same order; the two __constant__ values the reference sets
 * beforehand (c_jmax through copy_jmax_constant, GPU/dipole_GPU.h:14, and dip_stride_1
 * through copy_dipole_constant, :15) are the trailing arguments jmax and dip_stride.
 * Writes half_ls[startF_idx + f], 0 <= f < dimenF, for the F whose vibrational index lies
 * in [startFblock, endFblock); other entries are untouched.  Device pointers; asynchronous
 * on `stream` (a cudaStream_t, NULL = legacy default stream).  Results are bit-identical to
 * the reference kernel (same operations in the same order per output element). */
gain_status gain_hls_kblock(int dimenF, int dimenI, int jI, int jF, int kF,
                            const int* tauI, const int* tauF, const int* icorrI, const int* icorrF,
                            int startF_idx, int startI_idx, int startFblock, int endFblock,
                            int ncontrF, int kFBlocksize, const int* kblock_size,
                            const double* dipole_me, const double* vector, const double* threej,
                            double* half_ls, int jmax, int dip_stride, void* stream);

/* Rotational-symmetry (Euler) half line strength of one lower vector.
 * Replaces compute_gpu_half_linestrength_rotsym_ (GPU/dipole_GPU.h:38-41, GPU/dipole_GPU.cu:238-262,
 * kernel :641-723) with the same arguments in the same order; the __constant__ dip_stride_1
 * becomes the trailing dip_stride.  For every F (0 <= F < dimenF) whose vibrational index
 * icorrF[F] lies in [startFblock, endFblock):
 *   half_ls[F] = sum_I vector[I] sum_d wigner[d + 3 (ktauI[I] + nlevelI (ktauF[F] + nlevelF (kI[I] + sym_max_degen kF[F])))]
 *                * dipole_me[(icorrF[F] - startFblock) + icorrI[I] ncontrF + d ncontrF dip_stride],
 * where k holds the degeneracy index and ktau the rotational level index of each primitive
 * (TroveClasses/TroveBasisSet.cpp:480-483); other entries are untouched.  Device pointers;
 * asynchronous on `stream`.  Results are bit-identical to the reference kernel. */
gain_status gain_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int sym_max_degen,
                            const int* kI, const int* kF, const int* ktauI, const int* ktauF,
                            const int* icorrI, const int* icorrF, int startFblock, int endFblock,
                            int ncontrF, const double* dipole_me, const double* wigner,
                            const double* vector, double* half_ls, int dip_stride, void* stream);

/* Symmetry-adapted -> primitive expansion of one vector.
 * Replaces transform_vector_primitive (GPU/dipole_GPU.h:19, GPU/dipole_GPU.cu:137-156,
 * kernel :859-889): vec[r] = sum_{i<N[irow]} vecI[iterm+i] * repres[iterm+i + idegI*Ntot + ib*sdeg*Ntot]
 * with irow = icontr[r], ib = icontr[r+dimenI], iterm = ijterms[irow + igammaI*maxcoeff]. */
gain_status gain_expand(int dimenI, int igammaI, int maxcoeff, int idegI, int sdeg, int Ntot,
                        const int* ijterms, const int* icontr, const int* N, const double* repres,
                        const double* vecI, double* vec, void* stream);

/* result[0] = sum_i x[i]*y[i] (device pointers, device result).
 * Replaces the cublasDdot of GpuManager::ExecuteDotProduct (BaseClasses/GpuManager.cpp:741),
 * which runs in CUBLAS_POINTER_MODE_DEVICE (:202). */
gain_status gain_dot(int n, const double* x, const double* y, double* result, void* stream);

/* Same result as gain_dot (summed in another order: blocks of GAIN_DOT_NOALLOC_CHUNK
 * elements, then the block sums in block order) for callers that cannot allocate device
 * memory: host programs whose device memory is all handed out by their own pool allocator
 * (a framework's caching allocator that has already reserved the free memory, or a budget
 * that a direct cudaMalloc would break), and code on a path where an allocation's implicit
 * device synchronisation is not acceptable.  It calls no cudaMalloc/cudaFree and no
 * allocating library.  Its scratch is a fixed device array (GAIN_DOT_NOALLOC_MAX_N /
 * GAIN_DOT_NOALLOC_CHUNK partial sums plus a completion ticket, about 128 KB, held on every
 * device that loads the library until the process exits); n above GAIN_DOT_NOALLOC_MAX_N is
 * rejected with GAIN_ERR_INVALID_ARG.  The first call on each device looks up that array's
 * address (set-up, and again after the device's context was reset); make that first call
 * before any stream capture.  The scratch is shared by all calls on a device and keeps the
 * last call's contents: calls whose kernels overlap on the GPU race on it.
 * No counterpart in the reference (its dot product is the cuBLAS call gain_dot replaces). */
#define GAIN_DOT_NOALLOC_CHUNK 4096
#define GAIN_DOT_NOALLOC_MAX_N (16384LL * GAIN_DOT_NOALLOC_CHUNK)
gain_status gain_dot_noalloc(int n, const double* x, const double* y, double* result, void* stream);

/* Host: the Wigner-3j table GpuManager::InitializeAndTransferConstants builds
 * (BaseClasses/GpuManager.cpp:166-181, three_j -> TroveFortran/fort_func.f90:7-104):
 *   table[jI + kI(jmax+1) + (jF-jI+1)(jmax+1)^2 + (kF-kI+1)3(jmax+1)^2] = 3j(jI 1 jF; kI, kF-kI, -kF)
 * table holds 9 (jmax+1)^2 doubles.  Values are exact rationals rounded once, correctly. */
gain_status gain_threej_table(int jmax, double* table);

/* ======================= layer 2: the line-strength engine ========================= */

typedef struct gain_engine_s* gain_engine;

/* GpuManager ctor + InitializeAndTransferConstants (BaseClasses/GpuManager.cpp:69-213):
 * binds `device`, builds the 3j table for jmax on the device. nsym = number of irreducible
 * representations, maxdeg = largest degeneracy. */
gain_status gain_engine_create(int device, int jmax, int nsym, int maxdeg, gain_engine* out);
gain_status gain_engine_destroy(gain_engine e);

/* GpuManager::TransferBasisSet (BaseClasses/GpuManager.cpp:215-265): the primitive basis
 * of J (index jind): per function K, tau (ktau & 1), vibrational index; K-blocks.
 * Functions must be K-sorted (TroveClasses/TroveBasisSet.cpp:659-681). Host arrays, copied. */
gain_status gain_upload_basis(gain_engine e, int jind, int J, int dimen, const int* K,
                              const int* tau, const int* vib, const int* kblock_size,
                              const int* kstart);

/* GpuManager::TransferInflation (BaseClasses/GpuManager.cpp:381-422): expansion tables of
 * jind.  icontr[2*dimen], ijterms[maxcoeff*nsym]; per Gamma g: N[g][maxcoeff],
 * repres[g][Ntot[g]*sdeg[g]*matsize].  Host arrays, copied. */
gain_status gain_upload_inflation(gain_engine e, int jind, const int* icontr, const int* ijterms,
                                  int dimen, int maxcoeff, int matsize, const int* const* N,
                                  const double* const* repres, const int* Ntot, const int* sdeg);

/* GpuManager::TransferDipole (BaseClasses/GpuManager.cpp:499-526) for one DipolePiece
 * (BaseClasses/Dipole.h:9-15): piece[f-startF + i*ncontrF + d*N*ncontrF], d = 0..2,
 * N = Dipole::GetMaxContracts. Host array, copied. */
gain_status gain_upload_dipole(gain_engine e, const double* piece, int N, int startF, int endF,
                               int ncontrF);

/* The dipole as pieces of the upper vibrational index kept in HOST memory (TroveDipole's
 * blocks, TroveClasses/TroveDipole.cpp:85-112; each piece in the gain_upload_dipole layout
 * [3][N][endF-startF]), for N_v whose dipole does not fit the device.  Pieces are disjoint
 * and ascending.  Runs then loop over them as MultiGpuManager::ExecuteHalfLs loops over
 * dipole blocks (BaseClasses/MultiGpuManager.cpp:240-262, GpuManager::SwitchDipoleBlock
 * :481-496): one device buffer holds the piece in use; the split path accumulates the first
 * GEMM of every piece and runs the second GEMM once; the plain path sums the amplitudes of
 * one run per piece.  The host arrays must stay valid until the dipole is replaced or the
 * engine destroyed.  gain_adjoint_pair needs a single piece. */
gain_status gain_upload_dipole_pieces(gain_engine e, int npieces, const double* const* pieces, int N,
                                      const int* startF, const int* endF);

/* GpuManager::TransferWigner (BaseClasses/GpuManager.cpp:440-478): the rotational matrix
 * elements of the pair (J of jindI) -> (J of jindF), rot[d + 3 (lI + nlevelsI (lF + nlevelsF
 * (dI + maxdeg dF)))], d = 0..2 (the Wigner::rot layout the rotsym kernel reads,
 * GPU/dipole_GPU.cu:692).  Block pairs of these two J then run in the rotational-symmetry
 * form (GpuManager::ExecuteRotSymHalfLs, :547-610): M is dense in K, and each function's tau
 * is its rotational level index and K its degeneracy index (TroveBasisSet.cpp:480-483).
 * Host array, copied.  The batched engine handles non-degenerate levels (maxdeg 1). */
gain_status gain_upload_wigner(gain_engine e, int jindI, int jindF, int nlevelsI, int nlevelsF,
                               int maxdeg, const double* rot);

/* Eigenvectors of one (J, Gamma) block kept resident (the reference re-uploads one vector
 * per transition, GpuManager::UpdateEigenVector, :537-545): vecs[level*nsize + c].  Host
 * array (pinned memory transfers fastest) or device array, copied synchronously.  The copy
 * runs on the engine's own stream: a device array must be complete when the call is made
 * (work still queued on another stream that writes it is not waited for). */
gain_status gain_upload_eigvecs(gain_engine e, int jind, int gamma, int nlevels, int nsize,
                                const double* vecs);

/* Free the device copy of one (J, Gamma) block's eigenvectors (waits for the engine's queued
 * work).  For block sets larger than the device: upload the blocks a set of pairs needs, run
 * them, release, go on.  Plans that read the block re-capture on their next run (and fail
 * there with GAIN_ERR_NOT_READY until it is uploaded again).  No counterpart in the reference. */
gain_status gain_release_eigvecs(gain_engine e, int jind, int gamma);

/* As gain_upload_eigvecs, but from page-locked host memory the copy is only queued (on the
 * engine's copy stream) and the call returns at once; the next gain_run_pair orders every
 * read of these vectors after the copy, so the upper vectors of a pair stream in while the
 * lower side is computed.  vecs must stay unchanged until that gain_run_pair returns.  From
 * pageable memory it is the synchronous upload.  No counterpart in the reference. */
gain_status gain_upload_eigvecs_async(gain_engine e, int jind, int gamma, int nlevels, int nsize,
                                      const double* vecs);

typedef enum gain_path {
    GAIN_PATH_PLAIN_FP64 = 0,   /* the reference's method: half_ls per lower state, GEMV */
    GAIN_PATH_SPLIT = 1         /* Ozaki-sliced BF16 tcgen05 GEMMs + FP64 refinement */
} gain_path;

/* One block pair: rows = lower levels of (jindI, gammaI), columns = upper levels of
 * (jindF, gammaF).  Level lists are host arrays of level indices. */
typedef struct gain_pair_job {
    int jindI, gammaI, jindF, gammaF;
    int nlower;
    const int* lower_levels;
    int nupper;
    const int* upper_levels;
} gain_pair_job;

/* Certification of the split path: every output carries a rigorous error bound computed
 * from per-row norms.  Each half-line-strength entry (first GEMM) must be within the
 * worst-case rounding bound of an FP64 dot product of the same rows ("FP64-grade"); each
 * amplitude (second GEMM) within max(tol |amp|, that FP64 bound).  Outputs that fail (or
 * whose exact-accumulation certificate fails) are recomputed in FP64.  Every amplitude is
 * therefore within tol or within the reference FP64 method's own worst-case bound. */
typedef struct gain_split_opts {
    double tol;       /* relative tolerance on each amplitude (0 -> 4.5e-9, so that
                         S = amp^2 meets 1e-8) */
    int slices;       /* digits per operand of the amplitude GEMM (0 -> 49 bits; the
                         rotational-dipole GEMM always keeps 56 bits) */
    int beta;         /* bits per digit, 2..8 (0 -> 7) */
    int kchunks;      /* inner-dimension chunks for exact FP32 accumulation (0 -> auto) */
    double s_floor;   /* certification domain: lines with S >= s_floor * S_max must meet tol
                         (0 -> 1e-10, the domain of the headline accuracy requirement) */
} gain_split_opts;

typedef struct gain_stats {
    double device_ms;           /* device time of the last run (CUDA events) */
    long long rows, cols;       /* lower x upper amplitudes computed */
    long long refined;          /* split path: amplitudes recomputed in FP64 */
    long long uncertified;      /* split path, information: refined lines with S >= s_floor S_max
                                   whose FP64 bound itself exceeds tol |amp| (the reference's
                                   FP64 method cannot certify them either) */
    long long uncertified_weak; /* the same below s_floor S_max (outside the accuracy domain) */
    long long inexact;          /* split path: first-GEMM entries recomputed in FP64 (exactness
                                   certificate failed or bound above the FP64 bound) */
    double amp_max;             /* split path: largest |amplitude| of the run */
    int beta1, slices1, chunks1;  /* first GEMM (lower vectors x rotational-dipole matrix) */
    int beta2, slices2, chunks2;  /* second GEMM (half line strengths x upper vectors) */
    int products1, products2;   /* BF16 digit products per GEMM */
    int kernel_launches;        /* kernels launched by the last run */
    double gemm1_ms, gemm2_ms;  /* device time of the two tensor-core GEMMs */
    double tensor_flops;        /* BF16 MMA flops issued by the two GEMMs (whole tiles, padding
                                   included; the first GEMM counts its last dipole piece) */
} gain_stats;

/* Adjoint of one block pair (no counterpart in the reference): for a loss L over the line
 * strengths S = amp^2 of the pair, given dL_dS[l*nupper + u] (host, job order), ADD dL/dmu to
 * dL_dmu (host, the uploaded dipole piece's layout: [d][vibI][vibF - startF], 3 N ncontrF
 * doubles).  It runs the pair's FP64 forward (the plain path, so gain_fetch_amp returns its
 * amplitudes) and the adjoint chain in FP64: dL/damp = 2 amp dL/dS, dL/dH = dL/damp U,
 * dL/dh = T_F dL/dH, dL/dM = dL/dh^T v and the scatter of dL/dM into mu through the half line
 * strength's per-element factors (K-block or rotational-symmetry form).  Non-degenerate
 * symmetries (sdeg 1 on both sides; gain_adjoint_pair_degenerate takes the others). */
gain_status gain_adjoint_pair(gain_engine e, const gain_pair_job* job, const double* dL_dS,
                              double* dL_dmu, gain_stats* stats);

/* Arithmetic of the adjoint chain. */
typedef enum {
    GAIN_ADJOINT_FP64 = 0,   /* every product and sum in FP64 (gain_adjoint_pair) */
    GAIN_ADJOINT_FP32 = 1,   /* G, dL/dH, dL/dh, the lower vectors and the dL/dmu sums in FP32; the
                                FP64 amplitudes, eigenvectors and expansion tables are rounded to
                                FP32 as they are read; dL_dmu is still accumulated in double */
    GAIN_ADJOINT_SPLIT = 2   /* both products on the tensor cores as digit GEMMs (the split
                                path's Ozaki digits, 48 bits, exact accumulation, FP64
                                recombination; entries whose exactness certificate fails are
                                recomputed in FP64): dL/dH = G U over the upper states, and the
                                batched outer product dL/dM = sum_b dh_b v_b^T over the band of
                                the rotational-dipole matrix (|K_I - K_F| <= 1, or all K in the
                                rotational-symmetry form), then the FP64 scatter into dL/dmu.
                                Without the job's amplitudes from the last run it runs the split
                                forward (half line strengths recomputed, nothing per transition
                                kept from an earlier forward). */
} gain_adjoint_precision;

/* gain_adjoint_pair in the given precision. */
gain_status gain_adjoint_pair_prec(gain_engine e, const gain_pair_job* job, const double* dL_dS,
                                   double* dL_dmu, gain_adjoint_precision prec, gain_stats* stats);

/* Compute amplitudes amp[l][u] = <upper u | mu . rot | lower l> for one block pair into an
 * engine-owned device matrix (row-major; its pointer and leading dimension come from
 * gain_pair_amp_device).  Blocks on completion.  opts may be NULL (defaults).  stats may be
 * NULL. */
gain_status gain_run_pair(gain_engine e, const gain_pair_job* job, gain_path path,
                          const gain_split_opts* opts, gain_stats* stats);

/* A plan of block pairs over several engines of one device.  Each engine keeps its own
 * stream and buffers, so the jobs of different engines overlap on the GPU (small pairs leave
 * most SMs idle one at a time).  Every engine must hold the uploads the jobs need (bases,
 * expansion tables, dipole, eigenvectors).  One host thread per engine takes the largest
 * remaining job (the calling thread drives engines[0]) and runs gain_run_pair on it; then
 * on_done(user, job, engine, status), when given, is called from that thread, and the
 * engine's amplitudes (gain_fetch_amp, gain_pair_lines, ...) are that job's until it returns.
 * stats, when given, receives each job's stats at its index.  After a failure no further job
 * starts; the first failing status is returned, its message names the job. */
typedef void (*gain_job_done_fn)(void* user, int job, gain_engine engine, gain_status status);
gain_status gain_run_plan(gain_engine* engines, int n_engines, const gain_pair_job* jobs, int n_jobs,
                          gain_path path, const gain_split_opts* opts, gain_job_done_fn on_done, void* user,
                          gain_stats* stats);

/* ----------------------------------------------------------------------------------------
 * Grouped plans: many block pairs as ONE unit on one engine (the batched form of
 * main.cpp:238-342's loop over (J'', Gamma'') -> (J', Gamma') pairs and their lower states;
 * no counterpart in the reference, which launches per lower state and per transition,
 * BaseClasses/GpuManager.cpp:645-746).  The split path of every job runs as
 *   the digits of all jobs' lower and upper eigenvectors        (one launch per slicing
 *                                                                kernel; jobs of one block
 *                                                                share its digits)
 *   ONE persistent grouped tensor-core launch of the first GEMM over the tiles of all jobs
 *   per-job FP64 refinement of H (concurrent streams), then the digits of all jobs' H
 *   ONE persistent grouped tensor-core launch of the second GEMM over all jobs' tiles
 *   per-job FP64 refinement of the amplitudes                   (concurrent streams)
 * captured once into a CUDA graph and replayed by gain_plan_run.  The tiles of each grouped
 * launch are dealt to the persistent CTAs in list order, each to the first free one, with
 * the jobs with the costliest tiles (k-blocks x digit products) first, so block pairs of
 * very uneven sizes share one launch.  Each job keeps its own device buffers; the engine's
 * uploads (bases, expansion tables, dipole, eigenvectors) must hold every job's inputs.  Jobs are non-degenerate (components 0, 0) with a single dipole
 * piece.  After gain_plan_run, gain_plan_select makes one job's amplitudes the engine's last
 * run (for gain_fetch_amp, gain_pair_lines*, gain_pair_lines_text*, ...).
 *
 * Re-running after new eigenvectors of the same sizes were uploaded replays the same graph;
 * when inputs moved (a re-allocated eigenvector buffer, new dipole, bases or tables) the
 * plan is prepared and captured anew on its next run.  Destroy plans before their engine. */
typedef struct gain_plan_s* gain_plan;

/* gain_plan_create flags */
#define GAIN_PLAN_AUTOTUNE 1   /* choose the tile shape (CTA pairs or single CTAs) and, per size
                                  class of the second GEMM's inner dimension, its digit
                                  configuration (8-bit x 6 or 7-bit x 7) by timing the plan's
                                  candidates on first use; the choice is cached per plan shape
                                  for the process */

typedef struct gain_plan_stats {
    double device_ms;            /* the graph replay (CUDA events around it) */
    double gemm1_ms, gemm2_ms;   /* the two grouped GEMM launches inside it */
    long long transitions;       /* sum over jobs of lower x upper levels */
    long long refined;           /* H entries and amplitudes recomputed in FP64, all jobs */
    long long uncertified;       /* as gain_stats.uncertified, all jobs */
    int jobs, failed_jobs;
    int graph_nodes;             /* nodes of the captured graph */
    int kernel_launches;         /* kernel nodes among them */
    int gemm1_tiles, gemm2_tiles;/* tiles of the two grouped launches (empty slots excluded) */
    int units;                   /* persistent CTAs (CTA pairs) of each grouped launch */
    int pair;                    /* 1: 256 x 128 tiles on CTA pairs; 0: 128 x 128 tiles */
    int captures;                /* graph captures so far */
    int tuned;                   /* 1: the configuration came from the autotuner */
    double tune_ms;              /* wall time the autotuner spent (first use) */
    double tensor_flops;         /* BF16 MMA flops of the two grouped launches (whole tiles) */
    int beta2[4], slices2[4];    /* second-GEMM digits per size class of its inner dimension K:
                                    K <= 2048, <= 8192, <= 16384, above (0: class absent) */
    double digits_ms;            /* before the first GEMM: expansions and eigenvector digits */
    double middle_ms;            /* between the GEMMs: refinement of H, contraction, H digits */
    double refine_ms;            /* after the second GEMM: refinement of the amplitudes */
    int shared_lower;            /* jobs reading another job's lower digits (same lower block,
                                    levels, layout and first-GEMM digits) */
    int shared_upper;            /* jobs reading another job's upper digits */
} gain_plan_stats;

gain_status gain_plan_create(gain_engine e, const gain_pair_job* jobs, int n_jobs, const gain_split_opts* opts,
                             int flags, gain_plan* out);
/* Run (replay) the plan; job_stats[n_jobs] (may be NULL) receives each job's rows, cols and
 * refinement counts, stats (may be NULL) the plan's.  Returns the first failing job's status
 * (a refinement list that overflowed: GAIN_ERR_TOL_NOT_MET; a bounded device wait that gave
 * up: GAIN_ERR_TIMEOUT); the other jobs' amplitudes stay valid. */
gain_status gain_plan_run(gain_plan p, gain_stats* job_stats, gain_plan_stats* stats);
/* Make job's amplitudes (of the last gain_plan_run) the engine's last run. */
gain_status gain_plan_select(gain_plan p, int job);
/* Device pointer and leading dimension of job's amplitudes (valid until the next run). */
gain_status gain_plan_amp_device(gain_plan p, int job, const double** amp, int* ld);
gain_status gain_plan_destroy(gain_plan p);

/* Device pointer / leading dimension of the last run's amplitude matrix. */
gain_status gain_pair_amp_device(gain_engine e, const double** amp, int* ld);

/* Copy the last run's amplitudes to a host array amp[nlower*nupper] (row-major). */
gain_status gain_fetch_amp(gain_engine e, double* amp_host);

/* Intensity-block parameters (TroveClasses/TroveInput.cpp:239-326) the line assembly uses. */
typedef struct gain_line_params {
    double temperature;       /* TEMPERATURE */
    double q_part;            /* QSTAT */
    double zpe;               /* ZPE */
    double thresh;            /* THRESH_LINE */
    double freq_lo, freq_hi;  /* FREQ-WINDOW */
    double gnsF;              /* GNS of the upper Gamma */
    int ndegI, ndegF;         /* degeneracies of the pair's states; above 1 the lines combine the
                                 component slots of gain_run_pair_component (Output.cpp:78-91) */
    int reduced;              /* SYMMETRY REDUCED */
} gain_line_params;

/* Line strength S, Einstein A and intensity I of every amplitude of the last run
 * (Output::OutputLinestrength, BaseClasses/Output.cpp:52-112), on the device.  With
 * ndegI = ndegF = 1, S = amp^2 of the last run.  Otherwise S sums amp^2 over the component
 * slots (idegI < ndegI, idegF < ndegF, idegF outer) that gain_run_pair_component filled for
 * the last run's job, divides by ndegI and, when reduced and both states are degenerate,
 * multiplies by ndegI; the text's amplitude list holds those slots' amplitudes in that order.
 * energiesI/F are host arrays of the rows' / columns' energies.  keep[l*nupper+u] = 1 when
 * the reference would write the line (nu inside FREQ-WINDOW, nu >= 1e-40, A >= THRESH_LINE).
 * Host outputs (any may be NULL): S, A, I [nlower*nupper] doubles, keep [nlower*nupper]
 * bytes; n_lines = number kept. */
gain_status gain_pair_lines(gain_engine e, const gain_line_params* prm, const double* energiesI,
                            const double* energiesF, int jI, int jF, double* S, double* A,
                            double* I, unsigned char* keep, long long* n_lines);

/* gain_pair_lines without waiting: the line kernel is queued after the last run and its
 * copies into the host arrays (page-locked ones for a true overlap) run on a stream of their
 * own, so the engine's next uploads and run overlap them.  The arrays and *n_lines are
 * complete when gain_lines_wait returns; the next line assembly or text call on the engine,
 * and gain_engine_destroy, wait for them first. */
gain_status gain_pair_lines_async(gain_engine e, const gain_line_params* prm, const double* energiesI,
                                  const double* energiesF, int jI, int jF, double* S, double* A,
                                  double* I, unsigned char* keep, long long* n_lines);
/* Wait for the copies of the last gain_pair_lines_async (immediate when none is pending). */
gain_status gain_lines_wait(gain_engine e);

/* Line-list membership with THRESH_LINE > 0 (Output.cpp:95-96 drops a line when
 * A < THRESH_LINE): before the line assembly reads split-path amplitudes, every line whose A
 * lies within its certified error bound of THRESH_LINE is recomputed by the plain FP64 path
 * (the reference's method), for every component slot it combines, and those amplitudes
 * replace the split ones; the line assembly and text calls do this themselves.  This
 * returns how many lines the last line assembly or text call recomputed.  More than 65536
 * such lines fail that call with GAIN_ERR_TOL_NOT_MET.  No counterpart in the reference. */
gain_status gain_lines_threshold_refined(gain_engine e, long long* n_lines);

/* The intensity column of the line text (GAIN_TEXT_INTENSITY) is printed from the value the
 * reference's host code computes (Output.cpp:101-102 with the host C library's exp): a line
 * whose ten printed digits could change with the last bits of exp is evaluated on the host
 * and printed from that value; every other line's digits are the same either way.  This
 * returns how many lines the last text call evaluated on the host.  No counterpart in the
 * reference. */
gain_status gain_lines_intensity_host(gain_engine e, long long* n_lines);

/* Line-list text of the last run, built on the device: every line gain_pair_lines keeps,
 * written exactly as Output::OutputLinestrength prints it (BaseClasses/Output.cpp:99-111:
 * "%12.6f %8d %4d %4d <- %8d %4d %4d %16.9E " [intensity "%16.9E "] [ "[ " " %16.9E" " ] " ]
 * then " || \n"), in row-major order (lower state, then upper state).  Levels come from the
 * run's level lists and are printed + 1, gammaI/gammaF likewise; jI/jF are J values.  The
 * reference writes one line per Output call from an OpenMP loop over upper states
 * (main.cpp:286-339), so its order across upper states is that of its threads; each line's
 * bytes are what its sprintf/fprintf produce for the same doubles.  *text_bytes = size of the
 * text, *n_lines = lines written.  The text stays on the device until the next call. */
#define GAIN_TEXT_INTENSITY 1   /* compute_intensities: the intensity column */
#define GAIN_TEXT_AMPLITUDES 2  /* output_linestrengths: the "[ ... ]" amplitude list */
gain_status gain_pair_lines_text(gain_engine e, const gain_line_params* prm, const double* energiesI,
                                 const double* energiesF, int jI, int jF, int gammaI, int gammaF,
                                 int flags, unsigned long long* text_bytes, long long* n_lines);
/* gain_pair_lines_text with the text copied into out as it is formed: the copy of each
 * part overlaps the formatting of the next (page-locked out for that overlap).  cap must
 * hold the whole text; otherwise nothing is copied, *text_bytes holds its size and the call
 * returns GAIN_ERR_INVALID_ARG (the text stays on the device for gain_fetch_lines_text). */
gain_status gain_pair_lines_text_host(gain_engine e, const gain_line_params* prm, const double* energiesI,
                                      const double* energiesF, int jI, int jF, int gammaI, int gammaF,
                                      int flags, char* out, unsigned long long cap,
                                      unsigned long long* text_bytes, long long* n_lines);
/* Copy the text of the last gain_pair_lines_text call into out (cap >= text_bytes). */
gain_status gain_fetch_lines_text(gain_engine e, char* out, unsigned long long cap);
/* Device address and size of that text (valid until the next gain_pair_lines_text). */
gain_status gain_lines_text_device(gain_engine e, const char** text, unsigned long long* bytes);

/* Self-test of the bounded device waits the tensor-core GEMMs use (every mbarrier wait gives
 * up after a limit, raises the CTA's abort flag and reports GAIN_ERR_TIMEOUT): one wait on a
 * barrier nothing arrives on, limited to limit_ms (0 < limit_ms <= 1000).  Returns
 * GAIN_ERR_TIMEOUT when the wait gave up as it should; the engine stays usable. */
gain_status gain_selftest_bounded_wait(gain_engine e, double limit_ms);

/* The line-list conversions on their own, on the current device: values[i] printed with
 * "%<width>.<prec>E" (conv 'E', prec <= 17) or "%<width>.<prec>f" (conv 'f', prec <= 9) into
 * out + i*stride (no NUL), lens[i] = its length (the text is written only when it fits in
 * stride).  For checking the device conversion against the C library's printf. */
gain_status gain_format_values_device(const double* values, long long n, int conv, int width, int prec,
                                      char* out, int stride, int* lens);

/* ======================= host: state selection (BaseClasses/States.*) ============== */

/* One eigenstate (BaseClasses/States.h:327-346): J, index of J in the J list, symmetry,
 * degeneracy, level index inside its (J, Gamma) block, energy (cm^-1). */
typedef struct gain_state {
    double energy;
    int J, jind, gamma, ndeg, ilevel;
} gain_state;

/* The selection parameters of the INTENSITY block (TroveClasses/TroveInput.cpp:239-326).
 * isym_do[g] is derived as gns[g] >= 1e-15 (TroveInput.cpp:300-304). */
typedef struct gain_filters {
    int nsym;
    const double* gns;          /* [nsym] GNS */
    const int* isym_pairs;      /* [nsym] SELECTION */
    const int* igamma_pair;     /* [nsym] TroveInput::ComputeIGammaPair */
    const int* sym_degen;       /* [nsym] degeneracies */
    double erange_lower[2];     /* ENERGY LOW  lo hi */
    double erange_upper[2];     /* ENERGY UPPER lo hi */
    double freq_window[2];      /* FREQ-WINDOW lo hi */
    double zpe;                 /* ZPE */
    int maxJ;                   /* largest J of the run */
    int reduced;                /* SYMMETRY REDUCED */
    int symmetry_type;          /* 1 generic, 2 C3v/D3h, 3 Td (TroveInput.cpp:104-107) */
} gain_filters;

/* States::filter_lower / FilterLowerState (BaseClasses/States.cpp:46-49, States.h:61) */
int gain_filter_lower(const gain_filters* f, const gain_state* I);
/* States::FilterIntensity (BaseClasses/States.cpp:54-76) */
int gain_filter_intensity(const gain_filters* f, const gain_state* I, const gain_state* F);
/* States::DegeneracyFilter (BaseClasses/States.cpp:95-116) */
int gain_degeneracy_filter(const gain_filters* f, int gammaI, int gammaF, int idegI, int idegF);
/* States::GetTransitionDetails (BaseClasses/States.cpp:126-157) over a state table. */
gain_status gain_transition_details(const gain_filters* f, const gain_state* st, int n,
                                    int* num_initial, long long* num_trans, int* max_trans);

/* Block-pair plan of a state table: every (J'',Gamma'') -> (J',Gamma') pair that has at
 * least one transition, with the lower levels passing filter_lower and the upper levels
 * passing filter_upper (the separable part of FilterIntensity; the frequency window and
 * nu are applied per line by gain_pair_lines).  Pair p is
 *   pairs[4p .. 4p+3] = jindI, gammaI, jindF, gammaF,
 *   its lower levels  levels[offs[2p]   .. offs[2p+1]),
 *   its upper levels  levels[offs[2p+1] .. offs[2p+2]).
 * Call with pairs = NULL to get the sizes (n_pairs, n_levels); then with arrays of
 * 4 n_pairs, 2 n_pairs + 1 and n_levels ints. */
gain_status gain_plan_pairs(const gain_filters* f, const gain_state* st, int n, int* n_pairs,
                            int* pairs, int* offs, long long* n_levels, int* levels);

/* Degenerate symmetries (sdeg > 1 in the expansion tables).  Amplitudes of component idegI
 * of the lower states against component idegF of the upper states: the vectors expanded with
 * transform_vector_primitive's ideg (GPU/dipole_GPU.cu:137-156, 859-889), the reference's
 * linestrength[idegI + idegF * MaxDegen] (BaseClasses/GpuManager.cpp:733-746).  They become
 * the last run (gain_fetch_amp) and are kept in the engine's slot (idegI, idegF) for the line
 * assembly; a component run of another job empties the slots first.  gain_run_pair is
 * components (0, 0) without a slot. */
gain_status gain_run_pair_component(gain_engine e, const gain_pair_job* job, int idegI, int idegF,
                                    gain_path path, const gain_split_opts* opts, gain_stats* stats);
/* Every component pair of the job (idegI < sym_degen[gammaI], idegF < sym_degen[gammaF],
 * idegF outer) that passes gain_degeneracy_filter, through gain_run_pair_component (the
 * pairs main.cpp:238-342 and Output.cpp:78-85 compute).  stats sums the runs' times, counts
 * and launches. */
gain_status gain_run_pair_degenerate(gain_engine e, const gain_pair_job* job, const gain_filters* f,
                                     gain_path path, const gain_split_opts* opts, gain_stats* stats);
/* gain_adjoint_pair_prec for a pair of degenerate symmetries: dL_dS is the gradient over the
 * lines' S = sum over the component pairs passing gain_degeneracy_filter of amp^2, divided
 * by ndegI (times ndegI when filters->reduced and both states are degenerate), as
 * gain_pair_lines forms it; dL/dmu sums the adjoint chain of every such component pair, each
 * with its components' expansions.  A pair's forward amplitudes come from the last run or
 * the job's component slots when they hold it, else from the plain FP64 path. */
gain_status gain_adjoint_pair_degenerate(gain_engine e, const gain_pair_job* job, const gain_filters* f,
                                         const double* dL_dS, double* dL_dmu, gain_adjoint_precision prec,
                                         gain_stats* stats);

/* Text of one line exactly as Output.cpp:99-111 prints it, " || \n" included (without the
 * amplitude list unless namp > 0), through the C library's snprintf.  Returns the number of
 * characters written (excluding the NUL). */
int gain_format_line(char* buf, size_t cap, double nu, int indexF, int jF, int gammaF,
                     int indexI, int jI, int gammaI, double A, int with_intensity,
                     double intensity, const double* amps, int namp);
/* The same text through this library's own conversions (the code the device kernels run),
 * compiled for the host.  Returns the length, or minus the length needed when cap is too
 * small. */
int gain_format_line_native(char* buf, size_t cap, double nu, int indexF, int jF, int gammaF,
                            int indexI, int jI, int gammaI, double A, int with_intensity,
                            double intensity, const double* amps, int namp);
/* The length of that text from the value ranges alone where they fix it (the device's
 * length pass); equal to the length gain_format_line_native returns. */
long gain_line_length_native(double nu, int indexF, int jF, int gammaF, int indexI, int jI, int gammaI,
                             double A, int with_intensity, double intensity, const double* amps, int namp);
/* One value through those conversions: conv 'E' ("%<width>.<prec>E", prec <= 17) or 'f'
 * ("%<width>.<prec>f", prec <= 9); returns the length (minus the length needed when cap is
 * too small, 0 for a bad argument). */
int gain_format_value(char* buf, size_t cap, double x, int conv, int width, int prec);

#ifdef __cplusplus
}
#endif
#endif /* GAIN_LS_H */
