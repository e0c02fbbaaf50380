/* ORACLE (test infrastructure only): CPU restatement of the reference's FP64
 * line-strength path.  See gain_oracle.h for the cited reference functions.
 * Built with -ffp-contract=off so that the only fused multiply-adds are the explicit
 * fma() calls below, identically on x86-64 and aarch64. */
#include "gain_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------- double-double helpers (Dekker / Knuth error-free transforms) ------- */
typedef struct { double hi, lo; } dd;

static inline dd two_sum(double a, double b) {
    double s = a + b, bb = s - a;
    dd r = {s, (a - (s - bb)) + (b - bb)};
    return r;
}
static inline dd fast_two_sum(double a, double b) {
    double s = a + b;
    dd r = {s, b - (s - a)};
    return r;
}
static inline dd dd_from(double a) { dd r = {a, 0.0}; return r; }
static inline dd dd_mul_d(dd a, double b) {
    double p = a.hi * b;
    double e = fma(a.hi, b, -p);
    e += a.lo * b;
    return fast_two_sum(p, e);
}
static inline dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
static inline double dd_round(dd a) { return a.hi + a.lo; }

/* sign helper of the reference: 2*(~x & 1) - 1 == +1 for even x, -1 for odd x
 * (GPU/dipole_GPU.cu:459,509) */
static inline int parity_sign(int x) { return 2 * (~x & 1) - 1; }

/* half_ls of one upper primitive index irootF (one thread of the reference kernel). */
static double hls_one(int irootF, int dimenI, int jI, int jF, int kF,
                      const int* tauI_, const int* tauF_, const int* icorrI_, const int* icorrF_,
                      int startI_idx, int startFblock, int endFblock, int ncontrF,
                      const int* kblock_size_, const double* dipole_me, int dip_stride,
                      const double* vector, const double* threej, int jmax, int mode,
                      int* valid_out) {
    const int stride = ncontrF * dip_stride;                 /* :409 */
    int icontrF = icorrF_[irootF];
    const int tauF = tauF_[irootF] & 1;                      /* :425 */
    const int valid = (icontrF >= startFblock) && (icontrF < endFblock);   /* :429 */
    *valid_out = valid;
    if (!valid) return 0.0;
    icontrF -= startFblock;
    const int sigmaF = (kF % 3) * tauF;
    double acc = 0.0;
    dd acc_dd = dd_from(0.0);
    const int j1 = jmax + 1;
    for (int kI = (kF - 1 > 0 ? kF - 1 : 0); kI < kF + 2 && kI < jI + 1; kI++) {   /* :434-435 */
        const int kBlockSize = kblock_size_[kI];
        const double sq_factor = (kI * kF != 0) ? ORC_SQRT2 : 1.0;                 /* :439 */
        const int eq = (kF == kI), neq = (kF != kI);
        const double f3j = threej[jI + kI * j1 + (jF - jI + 1) * j1 * j1 + (kF - kI + 1) * j1 * j1 * 3];  /* :445 */
        for (int loc = 0; loc < kBlockSize; loc++) {
            const int irootI = startI_idx + loc;
            const int tauI = tauI_[irootI];                  /* :454 (not masked) */
            const int icI = icorrI_[irootI] * ncontrF;       /* :455 */
            const int sgnI = parity_sign((kI % 3) * tauI + kI);   /* :457-460 */
            double ls = vector[irootI];                      /* :462 */
            if (kF != kI) ls *= sq_factor;                   /* :464-466 */
            const double lsf = ls * f3j;                     /* :467 */
            if (lsf == 0.0) continue;                        /* :476 */
            const int tneq = (tauF != tauI);
            const int didx = 2 * eq + neq * (!tneq);         /* :490 */
            const int c = (tauF - tauI) * eq + (tauF - tauI) * (kF - kI) * neq * tneq - neq * (!tneq);  /* :492 */
            const double mu = dipole_me[icontrF + icI + didx * stride];    /* :495 */
            if (mode == ORC_REF) {
                const double t = lsf * (double)c;
                acc = fma(t * (double)sgnI, mu, acc);
            } else {
                if (c == 0) continue;
                dd t = dd_from(vector[irootI]);
                if (kF != kI) t = dd_mul_d(t, sq_factor);
                t = dd_mul_d(t, f3j);
                t.hi *= (double)(c * sgnI);
                t.lo *= (double)(c * sgnI);
                acc_dd = dd_add(acc_dd, dd_mul_d(t, mu));
            }
        }
        startI_idx += kBlockSize;                            /* :503-504 */
        if (startI_idx >= dimenI) break;
    }
    const double fs = (double)parity_sign(sigmaF);          /* :509 */
    return mode == ORC_REF ? acc * fs : dd_round(acc_dd) * fs;
}

void orc_hls_kblock(int dimenF, int dimenI, int jI, int jF, int kF,
                    const int* tauI, const int* tauF, const int* icorrI, const int* icorrF,
                    int startF_idx, int startI_idx, int startFblock, int endFblock, int ncontrF,
                    const int* kblock_size, const double* dipole_me, int dip_stride,
                    const double* vector, const double* threej, int jmax,
                    double* half_ls, int mode) {
#pragma omp parallel for schedule(static)
    for (int f = 0; f < dimenF; f++) {
        const int irootF = startF_idx + f;
        int valid;
        const double v = hls_one(irootF, dimenI, jI, jF, kF, tauI, tauF, icorrI, icorrF,
                                 startI_idx, startFblock, endFblock, ncontrF, kblock_size,
                                 dipole_me, dip_stride, vector, threej, jmax, mode, &valid);
        if (valid) half_ls[irootF] = v;                      /* :507-511 */
    }
}

/* The reference sums f_1 + f_2 + f_3 (f_d = w_d mu_d, GPU/dipole_GPU.cu:698-702) and adds
 * s_vector[i] times that sum to the accumulator.  The reference cubin evaluates it as
 *   t = fma(w0, mu0, w1 mu1); t = fma(w2, mu2, t); acc = fma(v, t, acc)
 * (identified bit for bit against that cubin's outputs on the rotsym golden vectors). */
static double rotsym_one(int irootF, int dimenI, int nlevelI, int nlevelF, int maxdeg, const int* kI,
                         const int* kF, const int* ktauI, const int* ktauF, const int* icorrI,
                         const int* icorrF, int startFblock, int ncontrF, const double* dipole_me,
                         int dip_stride, const double* wigner, const double* vector, int mode) {
    const size_t dstride = (size_t)ncontrF * (size_t)dip_stride;          /* :660 */
    const int icontrF = icorrF[irootF] - startFblock;                       /* :668,675 */
    const int lvlF = ktauF[irootF], degF = kF[irootF];
    double acc = 0.0;
    dd acc_dd = dd_from(0.0);
    for (int irootI = 0; irootI < dimenI; irootI++) {
        const size_t ic = (size_t)icorrI[irootI] * (size_t)ncontrF;         /* :679 */
        const double mu0 = dipole_me[icontrF + ic];                           /* :689-691 */
        const double mu1 = dipole_me[icontrF + ic + dstride];
        const double mu2 = dipole_me[icontrF + ic + 2 * dstride];
        const size_t w = (size_t)ktauI[irootI] * 3 + (size_t)lvlF * (size_t)nlevelI * 3 +
                         (size_t)kI[irootI] * (size_t)nlevelI * (size_t)nlevelF * 3 +
                         (size_t)degF * (size_t)maxdeg * (size_t)nlevelI * (size_t)nlevelF * 3;   /* :692 */
        const double w0 = wigner[w], w1 = wigner[w + 1], w2 = wigner[w + 2];
        const double v = vector[irootI];
        if (mode == ORC_DD) {
            dd sm = dd_add(dd_add(dd_mul_d(dd_from(w0), mu0), dd_mul_d(dd_from(w1), mu1)), dd_mul_d(dd_from(w2), mu2));
            acc_dd = dd_add(acc_dd, dd_mul_d(sm, v));
        } else {
            const double t = fma(w2, mu2, fma(w0, mu0, w1 * mu1));
            acc = fma(v, t, acc);
        }
    }
    return mode == ORC_DD ? dd_round(acc_dd) : acc;
}

void orc_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int maxdeg,
                    const int* kI, const int* kF, const int* ktauI, const int* ktauF,
                    const int* icorrI, const int* icorrF, int startFblock, int endFblock, int ncontrF,
                    const double* dipole_me, int dip_stride, const double* wigner,
                    const double* vector, double* half_ls, int mode) {
#pragma omp parallel for schedule(static)
    for (int f = 0; f < dimenF; f++) {
        const int icontrF = icorrF[f];
        if (icontrF < startFblock || icontrF >= endFblock) continue;        /* :674 */
        half_ls[f] = rotsym_one(f, dimenI, nlevelI, nlevelF, maxdeg, kI, kF, ktauI, ktauF, icorrI, icorrF,
                                startFblock, ncontrF, dipole_me, dip_stride, wigner, vector, mode);   /* :719 */
    }
}

void orc_half_ls(int jI, int jF, int dimenI, int dimenF,
                 const int* tauI, const int* tauF, const int* icorrI, const int* icorrF,
                 const int* kstartI, const int* kblockI, const int* kstartF, const int* kblockF,
                 int startFblock, int endFblock, int ncontrF,
                 const double* dipole_me, int dip_stride,
                 const double* prim_vector, const double* threej, int jmax,
                 double* half_ls, int mode) {
    memset(half_ls, 0, sizeof(double) * (size_t)dimenF);
    for (int kF = 0; kF < jF + 1; kF++) {
        orc_hls_kblock(kblockF[kF], dimenI, jI, jF, kF, tauI, tauF, icorrI, icorrF,
                       kstartF[kF], kstartI[kF - 1 > 0 ? kF - 1 : 0], startFblock, endFblock,
                       ncontrF, kblockI, dipole_me, dip_stride, prim_vector, threej, jmax,
                       half_ls, mode);
    }
}

void orc_expand(int dimenI, int igammaI, int maxcoeff, int idegI, int sdeg, int Ntot,
                const int* ijterms, const int* icontr, const int* N, const double* repres,
                const double* vecI, double* vec, int mode) {
    for (int r = 0; r < dimenI; r++) {
        const int irow = icontr[r];                          /* :871 */
        const int ib = icontr[r + dimenI];                   /* :873 */
        const int iterm = ijterms[irow + igammaI * maxcoeff];  /* :875 */
        const int nelem = N[irow];                           /* :877 */
        double acc = 0.0;
        dd acc_dd = dd_from(0.0);
        for (int i = 0; i < nelem; i++) {
            const int is = iterm + i;
            const double a = vecI[is], b = repres[is + idegI * Ntot + ib * sdeg * Ntot];  /* :882 */
            if (mode == ORC_REF) acc = fma(a, b, acc);
            else acc_dd = dd_add(acc_dd, dd_mul_d(dd_from(a), b));
        }
        vec[r] = mode == ORC_REF ? acc : dd_round(acc_dd);
    }
}

double orc_dot(int n, const double* x, const double* y, int mode) {
    if (mode == ORC_REF) {
        double acc = 0.0;
        for (int i = 0; i < n; i++) acc = fma(x[i], y[i], acc);
        return acc;
    }
    dd acc = dd_from(0.0);
    for (int i = 0; i < n; i++) acc = dd_add(acc, dd_mul_d(dd_from(x[i]), y[i]));
    return dd_round(acc);
}

int orc_run_pair(const orc_pair* p, int nthreads, int mode, double* amp) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    double* primI = (double*)malloc(sizeof(double) * (size_t)p->dimenI);
    double* hls = (double*)malloc(sizeof(double) * (size_t)p->dimenF);
    if (!primI || !hls) { free(primI); free(hls); return -1; }
    const int sdegI = p->sdegI > 0 ? p->sdegI : 1, sdegF = p->sdegF > 0 ? p->sdegF : 1;
    int err = 0;
    for (int l = 0; l < p->nlower; l++) {
        const double* vI = p->vec_lower + (size_t)l * p->NtotI;
        orc_expand(p->dimenI, p->gammaI, p->maxcoeffI, p->idegI, sdegI, p->NtotI, p->ijtermsI, p->icontrI,
                   p->NI, p->represI, vI, primI, mode);
        orc_half_ls(p->jI, p->jF, p->dimenI, p->dimenF, p->tauI, p->tauF, p->icorrI, p->icorrF,
                    p->kstartI, p->kblockI, p->kstartF, p->kblockF, p->startFblock, p->endFblock,
                    p->ncontrF, p->dipole_me, p->dip_stride, primI, p->threej, p->jmax, hls, mode);
#pragma omp parallel
        {
            double* primF = (double*)malloc(sizeof(double) * (size_t)p->dimenF);
            if (!primF) {
#pragma omp atomic write
                err = 1;
            } else {
#pragma omp for schedule(static)
                for (int u = 0; u < p->nupper; u++) {
                    const double* vF = p->vec_upper + (size_t)u * p->NtotF;
                    orc_expand(p->dimenF, p->gammaF, p->maxcoeffF, p->idegF, sdegF, p->NtotF, p->ijtermsF,
                               p->icontrF, p->NF, p->represF, vF, primF, mode);
                    amp[(size_t)l * p->nupper + u] = orc_dot(p->dimenF, primF, hls, mode);
                }
                free(primF);
            }
        }
        if (err) break;
    }
    free(primI);
    free(hls);
    return err ? -1 : 0;
}

int orc_line(const double* amp, const unsigned char* degmask, int maxdeg, int ndegI, int ndegF,
             int reduced, double energyI, double energyF, double zpe, int jI, int jF,
             double gnsF, double temperature, double q_part, double threshold,
             double* S_out, double* A_out, double* I_out) {
    double eI = energyI;
    const double nu = energyF - energyI;                   /* Output.cpp:63 */
    eI -= zpe;                                             /* :64 */
    if (nu < 1e-40) return 0;                              /* :65-66 */
    double ls = 0.0;
    for (int idegF = 0; idegF < ndegF; idegF++)
        for (int idegI = 0; idegI < ndegI; idegI++) {
            if (!degmask[idegI + idegF * maxdeg]) continue;
            const double l = amp[idegI + idegF * maxdeg];
            ls += l * l;                                   /* :82-83 */
        }
    ls /= (double)ndegI;                                   /* :89 */
    if (reduced && ndegF != 1 && ndegI != 1) ls *= (double)ndegI;   /* :90-91 */
    const double A = ORC_ACOEF * (double)(2 * jI + 1) * ls * fabs(nu) * fabs(nu) * fabs(nu);  /* :93 */
    if (A < threshold) return 0;                           /* :95 */
    const double beta = ORC_PLANCK * ORC_VELLGT / (ORC_BOLTZ * temperature);   /* :27 */
    const double I = ORC_CMCOEF * A * gnsF * (2.0 * (double)jF + 1.0)
                     * exp(-beta * eI) * (1.0 - exp(-beta * nu)) / (nu * nu * q_part);  /* :101-102 */
    *S_out = ls;
    *A_out = A;
    *I_out = I;
    return 1;
}

/* The line list of one block pair as the reference writes it: for every (lower r, upper c)
 * in row-major order, FilterIntensity's frequency window (BaseClasses/States.cpp:54-76),
 * then OutputLinestrength (BaseClasses/Output.cpp:52-112) with sprintf into a buffer and
 * fprintf "%s || \n".  amp[r*ld + c] is the line's amplitude (ndeg = 1).  Writes at most
 * cap bytes into out (out may be NULL to size); returns the text size, *n_lines the lines. */
long long orc_line_list(int rows, int cols, const double* amp, long ld, const double* eI, const double* eF,
                        const int* levI, const int* levF, int jI, int jF, int gammaI, int gammaF, double gnsF,
                        double temperature, double q_part, double zpe, double threshold, double freq_lo,
                        double freq_hi, int with_intensity, int with_amps, char* out, long long cap,
                        long long* n_lines) {
    const unsigned char one = 1;
    long long pos = 0, nl = 0;
    char buffer[1024], lsbuf[300];
    for (int r = 0; r < rows; ++r)
        for (int c = 0; c < cols; ++c) {
            const double nu = eF[c] - eI[r];
            if (!(nu >= freq_lo && nu <= freq_hi)) continue;
            const double a = amp[(long)r * ld + c];
            double S, A, I;
            if (!orc_line(&a, &one, 1, 1, 1, 0, eI[r], eF[c], zpe, jI, jF, gnsF, temperature, q_part, threshold,
                          &S, &A, &I))
                continue;
            lsbuf[0] = '\0';
            if (with_amps) sprintf(lsbuf + strlen(lsbuf), " %16.9E", a);
            sprintf(buffer, "%12.6f %8d %4d %4d <- %8d %4d %4d %16.9E ", nu, levF[c] + 1, jF, gammaF + 1,
                    levI[r] + 1, jI, gammaI + 1, A);
            if (with_intensity) sprintf(buffer + strlen(buffer), "%16.9E ", I);
            if (with_amps) sprintf(buffer + strlen(buffer), "[ %s ] ", lsbuf);
            char line[1100];
            const int n = snprintf(line, sizeof line, "%s || \n", buffer);
            if (out && pos + n <= cap) memcpy(out + pos, line, (size_t)n);
            pos += n;
            ++nl;
        }
    if (n_lines) *n_lines = nl;
    return pos;
}
