/* ORACLE (test infrastructure only).
 *
 * CPU restatement of the reference's FP64 line-strength path (GAIN-MPI).  Every function
 * names the reference code it follows.  The product library never links this; only the
 * tests, the smoke check and bench.py's CPU-baseline leg load it, as the checker.
 *
 * Accumulation modes:
 *   ORC_REF  -- the reference kernels' own operation order: ascending summation index,
 *               the accumulate step as one fused multiply-add (what nvcc emits for
 *               `acc += a*b` under its default -fmad=true).
 *   ORC_DD   -- compensated double-double evaluation of the same sums: the accurate
 *               FP64 answer, used as the error reference.
 */
#ifndef GAIN_ORACLE_H
#define GAIN_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_REF = 0, ORC_DD = 1 };

/* the reference's truncated constant, GPU/dipole_GPU.cu:24 and common/defines.h:23 */
#define ORC_SQRT2 0.70710678118
/* common/defines.h:17-24 */
#define ORC_PLANCK 6.62606896e-27
#define ORC_VELLGT 2.99792458e+10
#define ORC_BOLTZ 1.380658e-16
#define ORC_ACOEF 3.13618923e-7
#define ORC_CMCOEF 1.327209365e-12

/* One upper K-block of the half line strength:
 * device_compute_1st_half_ls_flipped_dipole_shared_block_nontrove, GPU/dipole_GPU.cu:392-515,
 * with the launch arguments of GpuManager::ExecuteKBlockHalfLs (BaseClasses/GpuManager.cpp:678-706).
 * dip_stride is the __constant__ dip_stride_1 (= Dipole::GetMaxContracts, GpuManager.cpp:514),
 * jmax the __constant__ c_jmax. */
void orc_hls_kblock(int dimenF, int dimenI, int jI, int jF, int kF,
                    const int* tauI, const int* tauF, const int* icorrI, const int* icorrF,
                    int startF_idx, int startI_idx, int startFblock, int endFblock, int ncontrF,
                    const int* kblock_size, const double* dipole_me, int dip_stride,
                    const double* vector, const double* threej, int jmax,
                    double* half_ls, int mode);

/* Whole half line strength of one (lower vector, J') pair: reset to zero
 * (GpuManager::ResetHalfLinestrength, :761-766) then one K-block per kF = 0..jF
 * (GpuManager::ExecuteKBlockHalfLs, :651-709). */
void orc_half_ls(int jI, int jF, int dimenI, int dimenF,
                 const int* tauI, const int* tauF, const int* icorrI, const int* icorrF,
                 const int* kstartI, const int* kblockI, const int* kstartF, const int* kblockF,
                 int startFblock, int endFblock, int ncontrF,
                 const double* dipole_me, int dip_stride,
                 const double* prim_vector, const double* threej, int jmax,
                 double* half_ls, int mode);

/* Rotational-symmetry (Euler) half line strength of one lower vector:
 * device_compute_1st_half_ls_flipped_dipole_shared_rotsym_nontrove, GPU/dipole_GPU.cu:641-723,
 * launched by compute_gpu_half_linestrength_rotsym_ (:238-262) from
 * GpuManager::ExecuteRotSymHalfLs (BaseClasses/GpuManager.cpp:547-610).  For every upper
 * primitive F whose vibrational index lies in [startFblock, endFblock):
 *   half_ls[F] = sum_I v[I] (w0 mu0 + w1 mu1 + w2 mu2),
 *   w_d = wigner[d + 3 (ktauI[I] + nlevelI (ktauF[F] + nlevelF (kI[I] + maxdeg kF[F])))],
 *   mu_d = dipole_me[(icorrF[F] - startFblock) + icorrI[I] ncontrF + d ncontrF dip_stride];
 * in rotsym mode ktau holds the rotational level index and k the degeneracy index
 * (TroveClasses/TroveBasisSet.cpp:480-483).  Other entries are untouched.  ORC_REF mode
 * forms the three-term sum as fma(w0, mu0, w1 mu1), then fma(w2, mu2, .), and accumulates it
 * with one fused multiply-add: the order of the reference cubin, bit for bit. */
void orc_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int maxdeg,
                    const int* kI, const int* kF, const int* ktauI, const int* ktauF,
                    const int* icorrI, const int* icorrF, int startFblock, int endFblock, int ncontrF,
                    const double* dipole_me, int dip_stride, const double* wigner,
                    const double* vector, double* half_ls, int mode);

/* Symmetry-adapted -> primitive expansion: device_expand_vectors, GPU/dipole_GPU.cu:859-889. */
void orc_expand(int dimenI, int igammaI, int maxcoeff, int idegI, int sdeg, int Ntot,
                const int* ijterms, const int* icontr, const int* N, const double* repres,
                const double* vecI, double* vec, int mode);

/* Dot product (the cublasDdot of GpuManager::ExecuteDotProduct, :741). */
double orc_dot(int n, const double* x, const double* y, int mode);

/* One block pair through the reference's plain FP64 loop order (main.cpp:238-342):
 * per lower state expand + half_ls, then per upper state expand + dot.  Only
 * non-degenerate symmetries (ndeg = 1) are handled here.  amp is [nlower][nupper].
 * nthreads > 1 parallelises the upper-state loop as main.cpp:292 does. */
typedef struct {
    int jI, jF, jmax;
    int dimenI, dimenF;
    const int *tauI, *tauF, *icorrI, *icorrF;
    const int *kstartI, *kblockI, *kstartF, *kblockF;
    /* expansion tables of the lower / upper (J, Gamma) */
    int gammaI, gammaF;
    int maxcoeffI, maxcoeffF, NtotI, NtotF;
    const int *ijtermsI, *icontrI, *NI;
    const double* represI;
    const int *ijtermsF, *icontrF, *NF;
    const double* represF;
    /* dipole piece */
    const double* dipole_me;
    int dip_stride, startFblock, endFblock, ncontrF;
    const double* threej;
    /* eigenvectors, rows of length NtotI / NtotF */
    int nlower, nupper;
    const double* vec_lower;
    const double* vec_upper;
    /* degenerate components (transform_vector_primitive's ideg) and the degeneracies of the
       two symmetries (0 reads as 1) */
    int idegI, idegF, sdegI, sdegF;
} orc_pair;

int orc_run_pair(const orc_pair* p, int nthreads, int mode, double* amp);

/* Line strength, Einstein A and intensity of one transition from its amplitudes
 * (Output::OutputLinestrength, BaseClasses/Output.cpp:52-112).  amp is the
 * [maxdeg*maxdeg] slot array indexed idegI + idegF*maxdeg; degmask marks the slots that
 * pass States::DegeneracyFilter.  Returns 0 when the line is not written (nu < 1e-40 or
 * A < threshold), 1 otherwise. */
int orc_line(const double* amp, const unsigned char* degmask, int maxdeg, int ndegI, int ndegF,
             int reduced, double energyI, double energyF, double zpe, int jI, int jF,
             double gnsF, double temperature, double q_part, double threshold,
             double* S_out, double* A_out, double* I_out);

/* The text the reference writes for one block pair's lines (row-major, ndeg = 1):
 * States.cpp:54-76 frequency window, Output.cpp:52-112 values and sprintf/fprintf.  out may
 * be NULL (sizing); returns the text size in bytes. */
long long orc_line_list(int rows, int cols, const double* amp, long ld, const double* eI, const double* eF,
                        const int* levI, const int* levF, int jI, int jF, int gammaI, int gammaF, double gnsF,
                        double temperature, double q_part, double zpe, double threshold, double freq_lo,
                        double freq_hi, int with_intensity, int with_amps, char* out, long long cap,
                        long long* n_lines);

#ifdef __cplusplus
}
#endif
#endif
