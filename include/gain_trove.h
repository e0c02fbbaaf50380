/* TROVE checkpoint ingestion for libgainls: the readers the reference uses to obtain the
 * inputs of its line-strength path, restated in C++ behind a C ABI.
 *
 *   j0eigen_quanta<J>.chk      primitive basis, J=0 correlation, symmetry tables
 *                              (TroveClasses/TroveBasisSet.cpp:27-292, 296-690, 692-710)
 *   j0_extfield.chk            vibrational dipole, flipped and split into pieces
 *                              (TroveClasses/TroveDipole.cpp:9-119, common/Util.cpp:89-109)
 *   j0eigen_descr<J>_<G>.chk   states of a (J, Gamma) block (TroveClasses/TroveStates.cpp:15-133)
 *   j0eigen_vectors<J>_<G>.chk eigenvector records (BaseClasses/EigenVector.cpp:126-140)
 *
 * The arrays these return are the arguments of gain_upload_basis, gain_upload_inflation,
 * gain_upload_dipole and gain_upload_eigvecs.  Every call returns a gain_status; a
 * malformed file is GAIN_ERR_INVALID_ARG with the reference's diagnostic in
 * gain_last_error_string(). */
#ifndef GAIN_TROVE_H
#define GAIN_TROVE_H

#include "gain_ls.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gain_trove_basis_s* gain_trove_basis;

/* Read j0eigen_quanta<J>.chk from dir (and j0eigen_quanta0.chk, the J=0 basis the
 * vibrational indices are correlated with).  nsym symmetries of degeneracies sym_degen.
 * rotsym = 0: the K-block form (tau = ktau & 1, K-blocks from the K-sorted functions);
 * rotsym = 1: K holds the rotational degeneracy index and tau the level index, as the
 * reference stores them for ROTSYM EULER (TroveBasisSet.cpp:478-483). */
gain_status gain_trove_basis_read(const char* dir, int J, int nsym, const int* sym_degen, int rotsym,
                                  gain_trove_basis* out);
void gain_trove_basis_free(gain_trove_basis b);
/* dimen (Maxcontracts), maxcoeff (Maxsymcoeffs), matsize; Ntot[nsym] may be NULL. */
gain_status gain_trove_basis_info(gain_trove_basis b, int* J, int* dimen, int* maxcoeff, int* matsize,
                                  int* Ntot);
/* K, tau, vib [dimen]; kblock, kstart [J+1]; icontr [2*dimen] (icontr2icase);
 * ijterms [maxcoeff*nsym].  Any pointer may be NULL. */
gain_status gain_trove_basis_arrays(gain_trove_basis b, int* K, int* tau, int* vib, int* kblock, int* kstart,
                                    int* icontr, int* ijterms);
/* N [maxcoeff] and repres [Ntot*sdeg*matsize] of one symmetry. */
gain_status gain_trove_basis_repres(gain_trove_basis b, int gamma, int* N, double* repres);
/* gain_upload_basis + gain_upload_inflation of this basis as J index jind. */
gain_status gain_trove_basis_upload(gain_engine e, int jind, gain_trove_basis b);

typedef struct gain_trove_dipole_s* gain_trove_dipole;

/* Read j0_extfield.chk (Fortran unformatted records, gfortran sub-records over 2 GiB
 * included) and split it into pieces of the upper contracted index as the reference does
 * for a device with max_bytes of memory: num_blocks = bytes / max_bytes + 1, pieces of
 * ceil(ncontr / num_blocks) functions (single-precision ceil, as TroveDipole.cpp:52,85). */
gain_status gain_trove_dipole_read(const char* path, unsigned long long max_bytes, gain_trove_dipole* out);
void gain_trove_dipole_free(gain_trove_dipole d);
gain_status gain_trove_dipole_info(gain_trove_dipole d, int* ncontr, int* nblocks);
/* The piece of one block in the flipped layout [3][ncontr][ncontrF] (f - startF + i ncontrF
 * + k ncontr ncontrF), valid until gain_trove_dipole_free. */
gain_status gain_trove_dipole_block(gain_trove_dipole d, int block, int* startF, int* endF, int* ncontrF,
                                    const double** piece);

/* One state of a descr file (EigenStates, BaseClasses/States.h:8-25). */
typedef struct gain_trove_state {
    double energy;
    int irec;      /* record of its eigenvector */
    int ilevel;    /* level index inside the (J, Gamma) block */
    int krot, taurot;
    int rec_len;   /* dim_basis of the file: doubles per eigenvector record */
} gain_trove_state;

/* States of j0eigen_descr<J>_<gamma+1>.chk in dir that pass States::filter_state (the lower
 * or the upper energy window and isym_do of f; BaseClasses/States.cpp:41-53), in file
 * order.  Call with out = NULL to count; *dim_basis = the record length. */
gain_status gain_trove_states_read(const char* dir, int J, int gamma, const gain_filters* f, int* n,
                                   gain_trove_state* out, int* dim_basis);

/* Eigenvector records records[0..n) of length rec_len from path into out[n*rec_len]
 * (record r at byte r*rec_len*8, EigenVector.cpp:126-140). */
gain_status gain_trove_vectors_read(const char* path, int rec_len, const int* records, int n, double* out);

#ifdef __cplusplus
}
#endif
#endif /* GAIN_TROVE_H */
