// TROVE checkpoint ingestion: the file formats the reference reads for its line-strength
// path, restated on the host (declarations and file map in include/gain_trove.h).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gain_trove.h"
#include "gain_internal.h"

using gain::set_error;

namespace {

std::string trim(const std::string& s) {
    const char* ws = " \t\r\n";
    const size_t a = s.find_first_not_of(ws);
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(ws);
    return s.substr(a, b - a + 1);
}

// Whitespace-separated integers / doubles of one line, strtol / strtod style.
struct Fields {
    const char* p;
    bool ok = true;
    explicit Fields(const std::string& s) : p(s.c_str()) {}
    long next_int() {
        char* e;
        errno = 0;
        const long v = strtol(p, &e, 0);
        if (e == p || errno) ok = false;
        p = e;
        return v;
    }
    double next_double() {
        char* e;
        const double v = strtod(p, &e);
        if (e == p) ok = false;
        p = e;
        return v;
    }
};

}  // namespace

// ------------------------------------------------------------------------------ basis
struct gain_trove_basis_s {
    int J = 0, nsym = 0, rotsym = 0;
    int ncases = 0, nlambdas = 0, ncontr = 0, nclasses = 0;   // Maxsymcoeffs, max_deg_size, Maxcontracts
    std::vector<int> nlam;                  // per case: index_deg(icase)%size1
    std::vector<int> cspace;                // [(nclasses+1) * ncases], 0-based
    std::vector<std::vector<int>> icoeffs;  // per case: [(nclasses+1) * nlam]
    std::vector<int> icontr2icase;          // [2 * ncontr]
    std::vector<int> icase2icontr;          // [ncases * nlambdas]
    int rot_ncases = 0, rot_nlambdas = 0;
    struct Rot { int j = 0, k = 0, tau = 0; };
    std::vector<Rot> rot_index;             // [rot_ncases * rot_nlambdas]
    int matsize = 0;
    std::vector<int> Ntot, sdeg;
    std::vector<std::vector<int>> N;        // per gamma [ncases]
    std::vector<std::vector<double>> repres;
    // derived (Correlate, ComputeijTerms)
    std::vector<int> K, ktau, vib, kblock, kstart, ijterms;
};

namespace {

// TroveBasisSet::ReadBasisSet (TroveBasisSet.cpp:27-292)
gain_status read_quanta(const std::string& path, int J, int nsym, const int* sym_degen, gain_trove_basis_s& b) {
    std::ifstream in(path);
    if (!in) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: cannot open %s", path.c_str());
    std::string line;
    auto next = [&](std::string& l) -> bool { return (bool)std::getline(in, l); };
    if (!next(line) || trim(line) != "Start Primitive basis set")
        return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad header %s", path.c_str());
    b.J = J;
    b.nsym = nsym;
    if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
    {
        Fields f(line);
        b.ncases = (int)f.next_int();
        b.nlambdas = (int)f.next_int();
        b.ncontr = (int)f.next_int();
        b.nclasses = (int)f.next_int();
        if (!f.ok || b.ncases <= 0 || b.nlambdas <= 0 || b.ncontr <= 0 || b.nclasses < 0)
            return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad sizes in %s", path.c_str());
    }
    const int nc1 = b.nclasses + 1;
    b.nlam.assign(b.ncases, 0);
    b.cspace.assign((size_t)nc1 * b.ncases, 0);
    b.icoeffs.assign(b.ncases, {});
    b.icontr2icase.assign(2 * (size_t)b.ncontr, 0);
    b.icase2icontr.assign((size_t)b.ncases * b.nlambdas, -1);
    int icontr = 0;
    for (int icase = 0; icase < b.ncases; ++icase) {
        if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
        Fields f(line);
        const int nl = (int)f.next_int();
        for (int i = 0; i < nc1; ++i) b.cspace[i + (size_t)icase * nc1] = (int)f.next_int() - 1;
        if (!f.ok || nl <= 0 || nl > b.nlambdas)
            return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad case %d in %s", icase + 1, path.c_str());
        b.nlam[icase] = nl;
        b.icoeffs[icase].assign((size_t)nc1 * nl, 0);
        for (int il = 0; il < nl; ++il) {
            if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
            Fields g(line);
            const int iroot = (int)g.next_int() - 1;
            for (int i = 0; i < nc1; ++i) b.icoeffs[icase][i + (size_t)il * nc1] = (int)g.next_int() - 1;
            if (!g.ok) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad line in %s", path.c_str());
            if (iroot != icontr || icontr >= b.ncontr)
                return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory] wrong indexing icontr = %d iroot = %d",
                                 icontr, iroot);
            b.icontr2icase[icontr] = icase;
            b.icontr2icase[icontr + b.ncontr] = il;
            b.icase2icontr[icase + (size_t)il * b.ncases] = icontr;
            ++icontr;
        }
    }
    if (icontr != b.ncontr) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory] wrong indexing");
    if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
    {
        Fields f(line);
        b.rot_ncases = (int)f.next_int();
        b.rot_nlambdas = (int)f.next_int();
        if (!f.ok || b.rot_ncases <= 0 || b.rot_nlambdas <= 0)
            return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad rot_index sizes in %s", path.c_str());
    }
    b.rot_index.assign((size_t)b.rot_ncases * b.rot_nlambdas, {});
    bool ended = false;
    while (next(line)) {
        if (trim(line) == "End Primitive basis set") {
            ended = true;
            break;
        }
        Fields f(line);
        const int icase = (int)f.next_int() - 1, il = (int)f.next_int() - 1;
        gain_trove_basis_s::Rot r;
        r.j = (int)f.next_int();
        r.k = (int)f.next_int();
        r.tau = (int)f.next_int();
        if (!f.ok || icase < 0 || icase >= b.rot_ncases || il < 0 || il >= b.rot_nlambdas)
            return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad rot_index line in %s", path.c_str());
        b.rot_index[icase + (size_t)il * b.rot_ncases] = r;
    }
    if (!ended) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: no basis footer in %s", path.c_str());
    if (!next(line) || trim(line) != "Start irreducible transformation")
        return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: wrong sym-footer");
    if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
    {
        Fields f(line);
        b.matsize = (int)f.next_int();
        if (!f.ok || b.matsize <= 0) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad mat_size");
    }
    if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
    b.Ntot.assign(nsym, 0);
    b.sdeg.assign(sym_degen, sym_degen + nsym);
    {
        Fields f(line);
        for (int g = 0; g < nsym; ++g) b.Ntot[g] = (int)f.next_int();
        if (!f.ok) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad Ntotal line");
    }
    b.N.assign(nsym, {});
    b.repres.assign(nsym, {});
    for (int g = 0; g < nsym; ++g) {
        if (b.Ntot[g] < 0 || b.sdeg[g] <= 0)
            return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad Ntotal / degeneracy of symmetry %d", g);
        b.N[g].assign(b.ncases, 0);
        for (int ic = 0; ic < b.ncases; ++ic) {
            if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
            Fields f(line);
            b.N[g][ic] = (int)f.next_int();
            if (!f.ok) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad N line");
        }
        const size_t nt = (size_t)b.Ntot[g], sd = (size_t)b.sdeg[g];
        b.repres[g].assign(nt * sd * b.matsize, 0.0);
        for (size_t ic = 0; ic < nt; ++ic)
            for (size_t id = 0; id < sd; ++id) {
                if (!next(line)) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: truncated %s", path.c_str());
                Fields f(line);
                for (int i = 0; i < b.matsize; ++i) b.repres[g][ic + id * nt + (size_t)i * nt * sd] = f.next_double();
                if (!f.ok) return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: bad repres line");
            }
    }
    if (!next(line) || trim(line) != "End irreducible transformation")
        return set_error(GAIN_ERR_INVALID_ARG, "[bset_contr_factory]: wrong irrep-footer");
    return GAIN_OK;
}

// TroveBasisSet::Correlate (TroveBasisSet.cpp:296-690) and ComputeijTerms (:692-710).  The
// J=0 match of each (case, lambda) is the first (jcase, jlambda) in the J=0 file order with
// equal vibrational classes and coefficients; a map keyed on those values finds it in one
// pass instead of the reference's nested search.
gain_status correlate(gain_trove_basis_s& b, const gain_trove_basis_s& j0) {
    const int nc = b.nclasses, nc1 = nc + 1, nc01 = j0.nclasses + 1;
    if (j0.nclasses < nc) return set_error(GAIN_ERR_INVALID_ARG, "[index_correlation] fewer classes at J=0");
    std::map<std::vector<int>, int> first;
    for (int jc = 0; jc < j0.ncases; ++jc)
        for (int jl = 0; jl < j0.nlam[jc]; ++jl) {
            std::vector<int> key(2 * (size_t)nc);
            for (int c = 0; c < nc; ++c) {
                key[c] = j0.cspace[(c + 1) + (size_t)jc * nc01];
                key[nc + c] = j0.icoeffs[jc][(c + 1) + (size_t)jl * nc01];
            }
            first.emplace(std::move(key), j0.icase2icontr[jc + (size_t)jl * j0.ncases]);
        }
    std::vector<int> corr((size_t)b.ncases * b.nlambdas, -1);
    for (int ic = 0; ic < b.ncases; ++ic)
        for (int il = 0; il < b.nlam[ic]; ++il) {
            std::vector<int> key(2 * (size_t)nc);
            for (int c = 0; c < nc; ++c) {
                key[c] = b.cspace[(c + 1) + (size_t)ic * nc1];
                key[nc + c] = b.icoeffs[ic][(c + 1) + (size_t)il * nc1];
            }
            auto it = first.find(key);
            if (it == first.end())
                return set_error(GAIN_ERR_INVALID_ARG,
                                 "[index_correlation] not found for J = %d -> problems with checkpoints?", b.J);
            corr[ic + (size_t)il * b.ncases] = it->second;
        }
    b.K.assign(b.ncontr, 0);
    b.ktau.assign(b.ncontr, 0);
    b.vib.assign(b.ncontr, 0);
    for (int ir = 0; ir < b.ncontr; ++ir) {
        const int ic = b.icontr2icase[ir], il = b.icontr2icase[ir + b.ncontr];
        const int jcontr = corr[ic + (size_t)il * b.ncases];
        if (jcontr < 0 || jcontr >= j0.ncontr)
            return set_error(GAIN_ERR_INVALID_ARG, "Error in root correlats %d %d", jcontr, j0.ncontr);
        b.vib[ir] = jcontr;
        const int ilevel = b.cspace[0 + (size_t)ic * nc1];
        const int ideg = b.icoeffs[ic][0 + (size_t)il * nc1];
        if (ilevel < 0 || ilevel >= b.rot_ncases || ideg < 0 || ideg >= b.rot_nlambdas)
            return set_error(GAIN_ERR_INVALID_ARG, "rotational index (%d, %d) outside rot_index", ilevel, ideg);
        const auto& r = b.rot_index[ilevel + (size_t)ideg * b.rot_ncases];
        b.ktau[ir] = 2 * r.k + r.tau;
        b.K[ir] = r.k;
        if (b.rotsym) {
            b.ktau[ir] = ilevel;
            b.K[ir] = ideg;
        }
    }
    b.kblock.assign(b.J + 1, 0);
    b.kstart.assign(b.J + 1, 0);
    if (b.rotsym) {   // no K-blocks in this form: counts per degeneracy index, for the upload
        for (int ir = 0; ir < b.ncontr; ++ir) {
            if (b.K[ir] > b.J)
                return set_error(GAIN_ERR_INVALID_ARG, "degeneracy index %d above J=%d", b.K[ir], b.J);
            ++b.kblock[b.K[ir]];
        }
        for (int k = 1; k <= b.J; ++k) b.kstart[k] = b.kstart[k - 1] + b.kblock[k - 1];
    } else {   // K-blocks of the K-sorted functions (:659-681)
        int last = 0, ksize = 0;
        for (int ir = 0; ir < b.ncontr; ++ir) {
            const int k = b.K[ir];
            b.ktau[ir] &= 1;
            if (k < last || k > b.J)
                return set_error(GAIN_ERR_INVALID_ARG, "basis of J=%d is not K-sorted (K=%d after K=%d)", b.J, k, last);
            if (k != last) {
                b.kblock[last] = ksize;
                b.kstart[k] = b.kstart[last] + ksize;
                ksize = 0;
                last = k;
            }
            ++ksize;
        }
        b.kblock[last] = ksize;
    }
    b.ijterms.assign((size_t)b.ncases * b.nsym, 0);
    for (int g = 0; g < b.nsym; ++g) {
        int n = 0;
        for (int it = 0; it < b.ncases; ++it) {
            b.ijterms[it + (size_t)g * b.ncases] = n;
            n += b.N[g][it];
        }
    }
    return GAIN_OK;
}

std::string join(const char* dir, const std::string& name) {
    std::string d = dir ? dir : ".";
    if (!d.empty() && d.back() != '/') d += '/';
    return d + name;
}

// ReadFortranRecord (common/Util.cpp:89-109): a gfortran sequential record, sub-records of
// 2^31 - 9 bytes with the continuation marker 0x80000009 when longer.  Returns the payload.
bool read_fortran_record(FILE* f, std::vector<char>& out) {
    out.clear();
    uint32_t m = 0;
    if (fread(&m, 4, 1, f) != 1) return false;
    const size_t chunk = 0x7fffffffu - 8u;
    while (m == 0x80000009u) {
        const size_t o = out.size();
        out.resize(o + chunk);
        if (fread(out.data() + o, 1, chunk, f) != chunk) return false;
        if (fread(&m, 4, 1, f) != 1 || fread(&m, 4, 1, f) != 1) return false;
    }
    const size_t o = out.size();
    out.resize(o + m);
    if (m && fread(out.data() + o, 1, m, f) != m) return false;
    return fread(&m, 4, 1, f) == 1;
}

}  // namespace

// ------------------------------------------------------------------------------ dipole
struct gain_trove_dipole_s {
    int ncontr = 0;
    struct Piece { int startF, endF, ncontrF; std::vector<double> data; };
    std::vector<Piece> pieces;
};

extern "C" {

gain_status gain_trove_basis_read(const char* dir, int J, int nsym, const int* sym_degen, int rotsym,
                                  gain_trove_basis* out) {
    gain::clear_error();
    if (!out || J < 0 || nsym <= 0 || !sym_degen) return set_error(GAIN_ERR_INVALID_ARG, "gain_trove_basis_read: bad argument");
    *out = nullptr;
    auto j0 = std::make_unique<gain_trove_basis_s>();
    j0->rotsym = rotsym;
    GAIN_TRY(read_quanta(join(dir, "j0eigen_quanta0.chk"), 0, nsym, sym_degen, *j0));
    GAIN_TRY(correlate(*j0, *j0));
    if (J == 0) {
        *out = j0.release();
        return GAIN_OK;
    }
    auto b = std::make_unique<gain_trove_basis_s>();
    b->rotsym = rotsym;
    GAIN_TRY(read_quanta(join(dir, "j0eigen_quanta" + std::to_string(J) + ".chk"), J, nsym, sym_degen, *b));
    GAIN_TRY(correlate(*b, *j0));
    *out = b.release();
    return GAIN_OK;
}

void gain_trove_basis_free(gain_trove_basis b) { delete b; }

gain_status gain_trove_basis_info(gain_trove_basis b, int* J, int* dimen, int* maxcoeff, int* matsize, int* Ntot) {
    gain::clear_error();
    if (!b) return set_error(GAIN_ERR_INVALID_ARG, "NULL basis");
    if (J) *J = b->J;
    if (dimen) *dimen = b->ncontr;
    if (maxcoeff) *maxcoeff = b->ncases;
    if (matsize) *matsize = b->matsize;
    if (Ntot) std::copy(b->Ntot.begin(), b->Ntot.end(), Ntot);
    return GAIN_OK;
}

gain_status gain_trove_basis_arrays(gain_trove_basis b, int* K, int* tau, int* vib, int* kblock, int* kstart,
                                    int* icontr, int* ijterms) {
    gain::clear_error();
    if (!b) return set_error(GAIN_ERR_INVALID_ARG, "NULL basis");
    if (K) std::copy(b->K.begin(), b->K.end(), K);
    if (tau) std::copy(b->ktau.begin(), b->ktau.end(), tau);
    if (vib) std::copy(b->vib.begin(), b->vib.end(), vib);
    if (kblock) std::copy(b->kblock.begin(), b->kblock.end(), kblock);
    if (kstart) std::copy(b->kstart.begin(), b->kstart.end(), kstart);
    if (icontr) std::copy(b->icontr2icase.begin(), b->icontr2icase.end(), icontr);
    if (ijterms) std::copy(b->ijterms.begin(), b->ijterms.end(), ijterms);
    return GAIN_OK;
}

gain_status gain_trove_basis_repres(gain_trove_basis b, int gamma, int* N, double* repres) {
    gain::clear_error();
    if (!b || gamma < 0 || gamma >= b->nsym) return set_error(GAIN_ERR_INVALID_ARG, "gain_trove_basis_repres: bad argument");
    if (N) std::copy(b->N[gamma].begin(), b->N[gamma].end(), N);
    if (repres) std::copy(b->repres[gamma].begin(), b->repres[gamma].end(), repres);
    return GAIN_OK;
}

gain_status gain_trove_basis_upload(gain_engine e, int jind, gain_trove_basis b) {
    gain::clear_error();
    if (!b) return set_error(GAIN_ERR_INVALID_ARG, "NULL basis");
    GAIN_TRY(gain_upload_basis(e, jind, b->J, b->ncontr, b->K.data(), b->ktau.data(), b->vib.data(), b->kblock.data(),
                               b->kstart.data()));
    std::vector<const int*> N(b->nsym);
    std::vector<const double*> R(b->nsym);
    for (int g = 0; g < b->nsym; ++g) {
        N[g] = b->N[g].data();
        R[g] = b->repres[g].data();
    }
    return gain_upload_inflation(e, jind, b->icontr2icase.data(), b->ijterms.data(), b->ncontr, b->ncases,
                                 b->matsize, N.data(), R.data(), b->Ntot.data(), b->sdeg.data());
}

// TroveDipole::InitDipole (TroveDipole.cpp:9-119)
gain_status gain_trove_dipole_read(const char* path, unsigned long long max_bytes, gain_trove_dipole* out) {
    gain::clear_error();
    if (!path || !out || max_bytes == 0) return set_error(GAIN_ERR_INVALID_ARG, "gain_trove_dipole_read: bad argument");
    *out = nullptr;
    std::unique_ptr<FILE, int (*)(FILE*)> f(fopen(path, "rb"), fclose);
    if (!f) return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] Error: checkpoint file of name %s not found", path);
    std::vector<char> rec;
    if (!read_fortran_record(f.get(), rec) || rec.size() < 20 || memcmp(rec.data(), "Start external field", 20) != 0)
        return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] Error: checkpoint file of name %s has bogus header", path);
    int32_t nc = 0;
    if (!read_fortran_record(f.get(), rec) || rec.size() < 4)
        return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] truncated %s", path);
    memcpy(&nc, rec.data(), 4);
    if (nc <= 0) return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] bad ncontr %d", nc);
    const size_t n = (size_t)nc, n2 = n * n;
    std::vector<double> temp(3 * n2);
    for (int i = 0; i < 3; ++i) {
        int32_t imu = 0;
        if (!read_fortran_record(f.get(), rec) || rec.size() < 4)
            return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] truncated %s", path);
        memcpy(&imu, rec.data(), 4);
        if (imu != i + 1)
            return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] has bogus imu - restore_vib_matrix_elements: %d /= %d",
                             imu, i + 1);
        if (!read_fortran_record(f.get(), rec) || rec.size() != n2 * sizeof(double))
            return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] component %d of %s: expected %zu bytes", i + 1, path,
                             n2 * sizeof(double));
        memcpy(temp.data() + i * n2, rec.data(), n2 * sizeof(double));
    }
    if (!read_fortran_record(f.get(), rec) || rec.size() < 18 || memcmp(rec.data(), "End external field", 18) != 0)
        return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] Error: checkpoint file of name %s has bogus footer", path);
    auto d = std::make_unique<gain_trove_dipole_s>();
    d->ncontr = nc;
    const unsigned long long bytes = 3ull * n2 * sizeof(double);
    const size_t nblocks = (size_t)(bytes / max_bytes) + 1;
    const size_t per = (size_t)ceil((float)n / (float)nblocks);
    for (size_t blk = 0; blk < nblocks; ++blk) {
        const size_t s = blk * per, e = std::min((blk + 1) * per, n);
        if (s > e) return set_error(GAIN_ERR_INVALID_ARG, "[read_dipole] %zu blocks of %zu functions overrun %zu", nblocks, per, n);
        gain_trove_dipole_s::Piece p;
        p.startF = (int)s;
        p.endF = (int)e;
        p.ncontrF = (int)(e - s);
        p.data.resize(3 * n * (e - s));
        for (size_t i = 0; i < n; ++i)   // flip: piece[f-startF + i ncontrF + k n ncontrF] = temp[i + f n + k n n]
            for (size_t fi = s; fi < e; ++fi)
                for (size_t k = 0; k < 3; ++k)
                    p.data[fi - s + i * (e - s) + k * n * (e - s)] = temp[i + fi * n + k * n2];
        d->pieces.push_back(std::move(p));
    }
    *out = d.release();
    return GAIN_OK;
}

void gain_trove_dipole_free(gain_trove_dipole d) { delete d; }

gain_status gain_trove_dipole_info(gain_trove_dipole d, int* ncontr, int* nblocks) {
    gain::clear_error();
    if (!d) return set_error(GAIN_ERR_INVALID_ARG, "NULL dipole");
    if (ncontr) *ncontr = d->ncontr;
    if (nblocks) *nblocks = (int)d->pieces.size();
    return GAIN_OK;
}

gain_status gain_trove_dipole_block(gain_trove_dipole d, int block, int* startF, int* endF, int* ncontrF,
                                    const double** piece) {
    gain::clear_error();
    if (!d || block < 0 || block >= (int)d->pieces.size())
        return set_error(GAIN_ERR_INVALID_ARG, "gain_trove_dipole_block: bad block");
    const auto& p = d->pieces[block];
    if (startF) *startF = p.startF;
    if (endF) *endF = p.endF;
    if (ncontrF) *ncontrF = p.ncontrF;
    if (piece) *piece = p.data.data();
    return GAIN_OK;
}

// TroveStates::ReadJGStates (TroveStates.cpp:15-133)
gain_status gain_trove_states_read(const char* dir, int J, int gamma, const gain_filters* f, int* n,
                                   gain_trove_state* out, int* dim_basis) {
    gain::clear_error();
    if (!f || !n || J < 0 || gamma < 0 || gamma >= f->nsym || !f->gns)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_trove_states_read: bad argument");
    // k_ind -> (K, tau) of the rotational levels: (0, J mod 2), then (k, 0), (k, 1) for k = 1..J
    std::vector<std::pair<int, int>> ktau_rot(1 + 2 * (size_t)J);
    ktau_rot[0] = {0, J % 2};
    for (int k0 = 1, r = 1; k0 <= J; ++k0)
        for (int t0 = 0; t0 <= 1; ++t0) ktau_rot[r++] = {k0, t0};
    const std::string path = join(dir, "j0eigen_descr" + std::to_string(J) + "_" + std::to_string(gamma + 1) + ".chk");
    std::ifstream in(path);
    if (!in) return set_error(GAIN_ERR_INVALID_ARG, "Error! couldn't open %s", path.c_str());
    std::string line;
    while (trim(line) != "Start Quantum numbers and energies")
        if (!std::getline(in, line)) return set_error(GAIN_ERR_INVALID_ARG, "Error! malformed descr file %s", path.c_str());
    std::getline(in, line);
    std::getline(in, line);
    if (!std::getline(in, line)) return set_error(GAIN_ERR_INVALID_ARG, "Error! malformed descr file %s", path.c_str());
    int dim = 0;
    {
        Fields fl(line);
        fl.next_int();   // nroots
        dim = (int)fl.next_int();
        if (!fl.ok || dim <= 0) return set_error(GAIN_ERR_INVALID_ARG, "Error! bad nroots/dim_basis line in %s", path.c_str());
    }
    const bool isym_do = f->gns[gamma] >= 1e-15;
    int count = 0;
    bool valid = false;
    while (std::getline(in, line)) {
        if (trim(line) == "End Quantum numbers and energies") {
            valid = true;
            break;
        }
        Fields fl(line);
        const int irec = (int)fl.next_int() - 1;
        const int ig = (int)fl.next_int() - 1;
        const int ilevel = (int)fl.next_int() - 1;
        fl.next_int();   // ideg
        const double energy = fl.next_double();
        if (!fl.ok) return set_error(GAIN_ERR_INVALID_ARG, "Error! bad state line in %s", path.c_str());
        if (ig != gamma) return set_error(GAIN_ERR_INVALID_ARG, "Gammas dont match in %s", path.c_str());
        const bool lower = (energy - f->zpe) <= f->erange_lower[1] && (energy - f->zpe) >= f->erange_lower[0];
        const bool upper = (energy - f->zpe) <= f->erange_upper[1] && (energy - f->zpe) >= f->erange_upper[0];
        if (!((lower || upper) && isym_do)) continue;   // States::filter_state
        const long k_ind = fl.next_int();
        if (!fl.ok || k_ind < 0 || k_ind > 2 * J)
            return set_error(GAIN_ERR_INVALID_ARG, "Error! bad rotational index in %s", path.c_str());
        if (out) {
            gain_trove_state& s = out[count];
            s.energy = energy;
            s.irec = irec;
            s.ilevel = ilevel;
            s.krot = ktau_rot[k_ind].first;
            s.taurot = ktau_rot[k_ind].second;
            s.rec_len = dim;
        }
        ++count;
    }
    if (!valid) return set_error(GAIN_ERR_INVALID_ARG, "Description file not complete! Footer not present!!!");
    *n = count;
    if (dim_basis) *dim_basis = dim;
    return GAIN_OK;
}

// EigenVector::ReadVectorFromFile (EigenVector.cpp:126-140): record r at r * rec_len doubles
gain_status gain_trove_vectors_read(const char* path, int rec_len, const int* records, int n, double* out) {
    gain::clear_error();
    if (!path || rec_len <= 0 || n < 0 || (n > 0 && (!records || !out)))
        return set_error(GAIN_ERR_INVALID_ARG, "gain_trove_vectors_read: bad argument");
    std::unique_ptr<FILE, int (*)(FILE*)> f(fopen(path, "rb"), fclose);
    if (!f) return set_error(GAIN_ERR_INVALID_ARG, "Could not open %s!!", path);
    const size_t len = (size_t)rec_len;
    for (int i = 0; i < n; ++i) {
        if (records[i] < 0) return set_error(GAIN_ERR_INVALID_ARG, "negative record %d", records[i]);
        if (fseeko(f.get(), (off_t)records[i] * (off_t)len * (off_t)sizeof(double), SEEK_SET) != 0 ||
            fread(out + (size_t)i * len, sizeof(double), len, f.get()) != len)
            return set_error(GAIN_ERR_INVALID_ARG, "record %d of %s is past its end", records[i], path);
    }
    return GAIN_OK;
}

}  // extern "C"
