// The C ABI of libgainls.so: kernel-level drop-ins, the engine that owns device memory,
// the plain FP64 and split-precision block-pair runs, line assembly and line text.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <queue>
#include <memory>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include <cstdlib>

#include "gain_internal.h"
#include "split.h"

namespace gain {

// ------------------------------------------------------------------ errors
namespace {
thread_local std::string g_last_error;
}

gain_status set_error(gain_status s, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}
void clear_error() { g_last_error.clear(); }
gain_status cuda_fail(cudaError_t e, const char* what) {
    (void)cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? GAIN_ERR_OOM : GAIN_ERR_CUDA, "%s: %s", what,
                     cudaGetErrorString(e));
}

namespace {

template <class T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    DevArray(DevArray&& o) noexcept : p(o.p), n(o.n) {
        o.p = nullptr;
        o.n = 0;
    }
    DevArray& operator=(DevArray&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevArray() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    gain_status alloc(size_t count) {
        if (p && count <= n) return GAIN_OK;
        release();
        if (!count) return GAIN_OK;
        cudaError_t e = cudaMalloc((void**)&p, sizeof(T) * count);
        if (e != cudaSuccess) {
            p = nullptr;
            return cuda_fail(e, "cudaMalloc");
        }
        n = count;
        return GAIN_OK;
    }
    gain_status upload(const T* h, size_t count) {
        GAIN_TRY(alloc(count));
        if (count) GAIN_CUDA(cudaMemcpy(p, h, sizeof(T) * count, cudaMemcpyHostToDevice));
        return GAIN_OK;
    }
    gain_status upload(const std::vector<T>& v) { return upload(v.data(), v.size()); }
    gain_status zero(cudaStream_t st, size_t count) {
        if (count) GAIN_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * count, st));
        return GAIN_OK;
    }
};

int round_up(int x, int m) { return (x + m - 1) / m * m; }

struct Basis {
    bool present = false;
    int J = 0, dimen = 0;
    std::vector<int> K, tau, vib, kblock, kstart;
    std::vector<int> lev;   // tau as uploaded (the rotational level index of the rotsym form)
    DevArray<int> dK, dtau, dvib, dkblock, dlev;
};

// Per symmetry and degenerate component of one J: derived structures of the expansion.
struct GammaMaps {
    bool built = false;
    std::vector<int> support;        // primitive functions the expansion touches, ascending
    std::vector<int> sup_start;      // [J+2] support grouped by K
    std::vector<int> csr_ptr, csr_col;   // transpose expansion: sym index -> primitives
    std::vector<double> csr_val;
    bool selection = false;          // every sym index is one primitive times a coefficient
    std::vector<int> sym_prim;
    std::vector<double> sym_coef;
    DevArray<int> d_support, d_sup_start, d_csr_ptr, d_csr_col;
    DevArray<double> d_csr_val;
};

struct Inflation {
    bool present = false;
    int dimen = 0, maxcoeff = 0, matsize = 0;
    std::vector<int> icontr, ijterms, Ntot, sdeg;
    std::vector<std::vector<int>> N;
    std::vector<std::vector<double>> repres;
    DevArray<int> dicontr, dijterms;
    std::vector<std::unique_ptr<DevArray<int>>> dN;
    std::vector<std::unique_ptr<DevArray<double>>> drepres;
    std::vector<std::unique_ptr<GammaMaps>> maps;
};

struct Eig {
    int nlevels = 0, nsize = 0;
    DevArray<double> d;
    // recorded on the copy stream after an asynchronous upload; every consumer's stream waits
    // on it before reading d (NULL until the first asynchronous upload)
    cudaEvent_t ready = nullptr;
    // the copy runs in two parts: rows [0, head_rows) are in place when ready_head fires
    cudaEvent_t ready_head = nullptr;
    int head_rows = 0;
    Eig() = default;
    Eig(const Eig&) = delete;
    Eig& operator=(const Eig&) = delete;
    ~Eig() {
        if (ready) cudaEventDestroy(ready);
        if (ready_head) cudaEventDestroy(ready_head);
    }
};

// Rotational matrix elements of one (J'', J') pair (the rotational-symmetry form):
// rot[d + 3 (lI + nI (lF + nF (dI + maxdeg dF)))], as GpuManager::TransferWigner stores them.
struct WignerTab {
    int nI = 0, nF = 0, maxdeg = 0;
    long version = 0;
    DevArray<double> rot;
};

struct StatsDev {
    DevArray<int> e, nnz;
    DevArray<float> l2, dn, dnv, rnv, inerr;
    gain_status alloc(size_t rows, int nch, bool with_inerr) {
        GAIN_TRY(e.alloc(rows));
        GAIN_TRY(nnz.alloc(rows));
        GAIN_TRY(l2.alloc(rows));
        GAIN_TRY(dn.alloc(rows * (size_t)nch));
        GAIN_TRY(dnv.alloc(rows * (size_t)split::MAX_SLICES));
        GAIN_TRY(rnv.alloc(rows * (size_t)split::MAX_SLICES));
        if (with_inerr) GAIN_TRY(inerr.alloc(rows));
        return GAIN_OK;
    }
    gain_status zero(cudaStream_t st, size_t rows, int nch, bool with_inerr) {
        GAIN_TRY(e.zero(st, rows));
        GAIN_TRY(nnz.zero(st, rows));
        GAIN_TRY(l2.zero(st, rows));
        GAIN_TRY(dn.zero(st, rows * (size_t)nch));
        GAIN_TRY(dnv.zero(st, rows * (size_t)split::MAX_SLICES));
        GAIN_TRY(rnv.zero(st, rows * (size_t)split::MAX_SLICES));
        if (with_inerr) GAIN_TRY(inerr.zero(st, rows));
        return GAIN_OK;
    }
    split::RowStats view(bool with_inerr, size_t row0 = 0, int nch = 0) {
        split::RowStats r;
        r.e = e.p + row0;
        r.nnz = nnz.p + row0;
        r.l2 = l2.p + row0;
        r.dn = dn.p + row0 * (size_t)nch;
        r.dnv = dnv.p + row0 * split::MAX_SLICES;
        r.rnv = rnv.p + row0 * split::MAX_SLICES;
        r.inerr = with_inerr ? inerr.p + row0 : nullptr;
        return r;
    }
};

// Split-path layout of one block pair (lower layout padded per K block to BK, upper layout
// padded per K block to BN so that no output tile straddles two upper K blocks).
struct PairLayout {
    int key[6] = {-1, -1, -1, -1, -1, -1};   // pair and components
    long dip_version = -1, wig_version = -1;
    int nI = 0, kpadI = 0, nF = 0, fpad = 0, W = 0;
    bool rotsym = false;
    std::vector<int> kpad_startI;   // [J_I + 2]
    std::vector<int> colposI, i_sym, i_prim;
    std::vector<double> i_coef;
    std::vector<int> colposF, f_sym, f_prim, band_k0, band_len;
    std::vector<double> f_coef;
    std::vector<std::pair<int, int>> fblocks;   // padded [start, end) of each upper K block
    DevArray<int> d_colposI, d_i_sym, d_i_prim, d_colposF, d_f_sym, d_f_prim, d_band_k0, d_band_len;
    DevArray<double> d_i_coef, d_f_coef, band;
    int beta1 = 0, s1 = 0, c1 = 0;
    DevArray<__nv_bfloat16> bandDig;
    StatsDev bandStats;
    CUtensorMap tmBand, tmBandPair;   // 128-row boxes; 64-row boxes for a CTA pair
    // an expansion that mixes primitives (not a selection): both GEMM1 layouts run over the
    // primitives the expansions touch; H = V T_I M is contracted with T_F before GEMM2,
    // whose inner dimension is then the nsymF symmetric functions padded to ntpad
    bool general = false;
    // an expansion that mixes primitives of one K only: GEMM1 stays over symmetric functions
    // and the band combines the primitive entries through both expansions
    bool symband = false;
    std::vector<int> fr_ptr, fr_col, ic_ptr, ic_col;   // per padded row / column: (primitive, coefficient)
    std::vector<double> fr_val, ic_val;
    DevArray<int> d_fr_ptr, d_fr_col, d_ic_ptr, d_ic_col;
    DevArray<double> d_fr_val, d_ic_val;
    int nsymF = 0, ntpad = 0;
    double sigmaF = 1.0, gamF = 0.0;      // ||T_F||_2 bound; FP64 contraction rounding factor
    std::vector<int> cF_ptr, cF_col;      // T_F^T as CSR over symmetric functions, columns in F layout
    std::vector<double> cF_val;
    DevArray<int> d_cF_ptr, d_cF_col, d_ident;
    DevArray<double> d_cF_val;
};

size_t layout_bytes(const PairLayout& L) {
    return L.band.n * sizeof(double) + L.bandDig.n * sizeof(__nv_bfloat16);
}

// Plain-path structures of one block pair.
struct PlainLayout {
    int key[6] = {-1, -1, -1, -1, -1, -1};   // pair and components
    std::vector<HlsCta> ctas;
    DevArray<HlsCta> d_ctas;
    DevArray<int> d_flist;
};

}  // namespace
}  // namespace gain

struct gain_engine_s {
    int device = 0;
    int jmax = 0, nsym = 0, maxdeg = 0;
    int num_sms = 0;
    cudaStream_t st = nullptr;
    cudaStream_t st2 = nullptr;   // upper-vector slicing, concurrent with the lower side
    cudaStream_t stc = nullptr;   // asynchronous eigenvector uploads
    cudaStream_t std2h = nullptr; // device-to-host copies of an asynchronous line assembly
    cudaEvent_t ev_lines = nullptr, ev_lines_d2h = nullptr;
    // kept-line count of the line assembly (apart from the run's counters, which the next run
    // zeroes while an asynchronous copy of this one may still be pending)
    gain::DevArray<unsigned long long> lcnt;
    bool lines_pending = false;     // gain_pair_lines_async copies still in flight
    long long* lines_nout = nullptr;   // their caller's n_lines
    cudaEvent_t ev[10] = {};
    // orders an asynchronous upload after the engine work that reads eigenvectors: recorded
    // at the end of every run (runs, plans, adjoints and line recomputations return only when
    // their work is done), so an upload need not wait for line kernels queued after a run
    cudaEvent_t ev_up = nullptr;
    bool ev_up_fresh = false;   // recorded after the last eigenvector reader (else record anew)
    std::vector<long> zkey_V, zkey_H, zkey_U;   // shape/layout the digit buffers were cleared for
    gain::DevArray<double> d3j;
    std::vector<gain::Basis> bases;
    std::vector<gain::Inflation> infl;
    gain::DevArray<double> dipole;
    int dipN = 0, startF = 0, endF = 0, ncontrF = 0;
    bool dip_present = false;
    long dip_version = 0;
    long struct_version = 0;   // bases and expansion tables (plans re-capture when it moves)
    // dipole pieces kept in host memory (gain_upload_dipole_pieces); runs loop over them
    struct HostPiece {
        const double* host;
        int startF, endF;
    };
    std::vector<HostPiece> pieces;
    int piece_loaded = -1;
    gain::DevArray<double> acc;   // amplitude / H accumulator of a multi-piece run
    std::map<std::pair<int, int>, std::unique_ptr<gain::WignerTab>> wigner;   // by (jindI, jindF)
    long wig_version = 0;
    std::map<std::pair<int, int>, std::unique_ptr<gain::Eig>> eig;

    // last run
    gain::DevArray<double> amp;
    int amp_rows = 0, amp_cols = 0;
    long amp_ld = 0;
    bool have_amp = false;
    std::vector<int> amp_job;   // job_key of amp: the pair, its level lists and components
    // split path: the certified absolute error bound of every amplitude (ld amp_ld); the line
    // assembly recomputes in FP64 the lines whose Einstein A lies within its bound of
    // THRESH_LINE (line-list membership)
    gain::DevArray<float> ampbnd;
    bool have_bnd = false;
    long long thresh_refined = 0;   // lines the last line assembly recomputed for THRESH_LINE
    // degenerate component slots of one job (gain_run_pair_component): [maxdeg^2][rows * cols]
    gain::DevArray<double> deg_amp;
    std::vector<int> deg_job;   // job_key (components 0, 0) of the slots
    unsigned deg_filled = 0;    // bit idegI + idegF * maxdeg per filled slot
    gain::DevArray<float> deg_bnd;   // the slots' amplitude bounds (0 for plain-path slots)
    // FP64 recomputation of lines near THRESH_LINE: flagged lines, level subsets, amplitudes
    gain::DevArray<int2> thr_list;
    gain::DevArray<unsigned int> thr_cnt;
    gain::DevArray<int> sub_lower, sub_upper;
    gain::DevArray<double> sub_amp, sub_acc;
    gain::DevArray<long long> sub_patch;
    // intensity column: lines whose intensity the host evaluates (see gain_pair_lines_text)
    gain::DevArray<gain::TextArgs::HardLine> hardLines;
    gain::DevArray<unsigned int> hardCount;
    gain::DevArray<long long> ovrIdx;
    gain::DevArray<double> ovrVal;
    gain::DevArray<double> pow10;   // 10^k, k = -300..300, correctly rounded (C library strtod)
    long long intensity_host = 0;
    long launches = 0;          // kernels this engine has launched (split path and band builds)
    void* readback = nullptr;   // page-locked area of a run's counter readbacks

    // work buffers
    gain::DevArray<int> d_lower, d_upper;
    gain::DevArray<double> primI, hprim, hsym;
    gain::DevArray<double> adj_dLdS, adj_G, adj_dH, adj_dh, adj_vp, adj_dmu;   // adjoint work space
    gain::DevArray<int> adj_iota, adj_tiles;
    // the tensor-core adjoint: transposed operands, digits, statistics, layout and GEMM lists
    gain::DevArray<double> adjs_UT, adjs_dhT, adjs_vpT, adjs_dM, adjs_dH;
    gain::DevArray<__nv_bfloat16> adjs_dig[4];
    gain::StatsDev adjs_st[4];
    gain::DevArray<int> adjs_fmap, adjs_imap, adjs_blo, adjs_bhi, adjs_err, adjs_umap;
    gain::DevArray<int2> adjs_flags;
    gain::DevArray<unsigned int> adjs_cnt;
    gain::DevArray<gain::split::Tile> adjs_tiles1, adjs_tiles2;
    gain::DevArray<gain::split::Prod> adjs_prods1, adjs_prods2;
    gain::DevArray<__nv_bfloat16> Vdig, Hdig, Udig;
    gain::StatsDev Vst, Hst, Ust;
    gain::DevArray<double> H, Hsym;   // H in the GEMM1 layout; contracted with a mixing expansion
    gain::DevArray<int> iota;
    gain::DevArray<float> rowerr;
    gain::DevArray<int2> flags1, flags2;
    gain::DevArray<unsigned int> counters;      // [0] nflags1 [1] nflags2
    gain::DevArray<unsigned long long> ull;     // [0] uncertified [1] nkeep
    gain::DevArray<int> err;
    gain::DevArray<gain::split::Tile> tiles1, tiles2;
    gain::DevArray<gain::split::Prod> prods1, prods2;
    gain::DevArray<double> lineS, lineA, lineI, eIdev, eFdev;
    gain::DevArray<unsigned char> lineKeep;
    gain::DevArray<uint32_t> textLens;
    gain::DevArray<unsigned long long> textBlocks;   // block offsets, then [nblocks] total, [nblocks+1] lines
    gain::DevArray<char> text;
    unsigned long long text_bytes = 0;
    bool have_text = false;

    // split-path layouts (band, its digits, padded index maps) per block pair, kept across runs
    std::map<std::array<int, 6>, std::shared_ptr<gain::PairLayout>> layouts;   // plans share them
    gain::PairLayout* cur = nullptr;   // the layout of the current run
    gain::PlainLayout plain;
};

namespace gain {
namespace {

constexpr int kMaxFlags = 1 << 22;

gain_status check_engine(gain_engine e) {
    if (!e) return set_error(GAIN_ERR_INVALID_ARG, "engine is NULL");
    GAIN_CUDA(cudaSetDevice(e->device));
    return GAIN_OK;
}

// The expansion of component ideg of Gamma g (transform_vector_primitive's ideg).
GammaMaps* gamma_maps(gain_engine e, int jind, int g, int ideg) {
    Basis& b = e->bases[jind];
    Inflation& inf = e->infl[jind];
    GammaMaps& m = *inf.maps[(size_t)g * e->maxdeg + ideg];
    if (m.built) return &m;
    const int d = inf.dimen;
    const int Ntot = inf.Ntot[g], sdeg = inf.sdeg[g];
    m.support.clear();
    m.sup_start.assign(b.J + 2, 0);
    std::vector<std::vector<std::pair<int, double>>> rows(Ntot);
    bool sel = true;
    for (int r = 0; r < d; ++r) {
        const int irow = inf.icontr[r], ib = inf.icontr[r + d];
        const int nel = inf.N[g][irow];
        if (nel <= 0) continue;
        m.support.push_back(r);
        if (nel != 1) sel = false;
        const int iterm = inf.ijterms[irow + g * inf.maxcoeff];
        for (int i = 0; i < nel; ++i) {
            const int s = iterm + i;
            const double coef = inf.repres[g][(size_t)s + (size_t)ideg * Ntot + (size_t)ib * sdeg * Ntot];
            rows[s].push_back({r, coef});
        }
    }
    for (int r : m.support) m.sup_start[b.K[r] + 1]++;
    for (int k = 0; k <= b.J; ++k) m.sup_start[k + 1] += m.sup_start[k];
    m.csr_ptr.assign(Ntot + 1, 0);
    m.csr_col.clear();
    m.csr_val.clear();
    m.sym_prim.assign(Ntot, -1);
    m.sym_coef.assign(Ntot, 0.0);
    for (int s = 0; s < Ntot; ++s) {
        std::sort(rows[s].begin(), rows[s].end());
        for (auto& pr : rows[s]) {
            m.csr_col.push_back(pr.first);
            m.csr_val.push_back(pr.second);
        }
        m.csr_ptr[s + 1] = (int)m.csr_col.size();
        if (rows[s].size() == 1) {
            m.sym_prim[s] = rows[s][0].first;
            m.sym_coef[s] = rows[s][0].second;
        } else {
            sel = false;
        }
    }
    m.selection = sel;
    if (m.d_support.upload(m.support) || m.d_sup_start.upload(m.sup_start) ||
        m.d_csr_ptr.upload(m.csr_ptr) || m.d_csr_col.upload(m.csr_col) || m.d_csr_val.upload(m.csr_val))
        return nullptr;
    m.built = true;
    return &m;
}

gain_status validate_job(gain_engine e, const gain_pair_job* j) {
    if (!j) return set_error(GAIN_ERR_INVALID_ARG, "job is NULL");
    const int nj = (int)e->bases.size();
    if (j->jindI < 0 || j->jindI >= nj || j->jindF < 0 || j->jindF >= nj)
        return set_error(GAIN_ERR_INVALID_ARG, "jind out of range");
    if (!e->bases[j->jindI].present || !e->bases[j->jindF].present)
        return set_error(GAIN_ERR_NOT_READY, "basis set of jind %d/%d not uploaded", j->jindI, j->jindF);
    if (!e->infl[j->jindI].present || !e->infl[j->jindF].present)
        return set_error(GAIN_ERR_NOT_READY, "expansion tables not uploaded");
    if (!e->dip_present) return set_error(GAIN_ERR_NOT_READY, "dipole not uploaded");
    if (j->gammaI < 0 || j->gammaI >= e->nsym || j->gammaF < 0 || j->gammaF >= e->nsym)
        return set_error(GAIN_ERR_INVALID_ARG, "gamma out of range");
    const int JI = e->bases[j->jindI].J, JF = e->bases[j->jindF].J;
    if (std::abs(JI - JF) > 1) return set_error(GAIN_ERR_INVALID_ARG, "|J' - J''| > 1");
    if (JI > e->jmax || JF > e->jmax) return set_error(GAIN_ERR_INVALID_ARG, "J above jmax");
    auto itI = e->eig.find({j->jindI, j->gammaI});
    auto itF = e->eig.find({j->jindF, j->gammaF});
    if (itI == e->eig.end() || itF == e->eig.end())
        return set_error(GAIN_ERR_NOT_READY, "eigenvectors of the pair not uploaded");
    if (j->nlower <= 0 || j->nupper <= 0 || !j->lower_levels || !j->upper_levels)
        return set_error(GAIN_ERR_INVALID_ARG, "empty level lists");
    for (int i = 0; i < j->nlower; ++i)
        if (j->lower_levels[i] < 0 || j->lower_levels[i] >= itI->second->nlevels)
            return set_error(GAIN_ERR_INVALID_ARG, "lower level %d out of range", j->lower_levels[i]);
    for (int i = 0; i < j->nupper; ++i)
        if (j->upper_levels[i] < 0 || j->upper_levels[i] >= itF->second->nlevels)
            return set_error(GAIN_ERR_INVALID_ARG, "upper level %d out of range", j->upper_levels[i]);
    if (itI->second->nsize != e->infl[j->jindI].Ntot[j->gammaI] ||
        itF->second->nsize != e->infl[j->jindF].Ntot[j->gammaF])
        return set_error(GAIN_ERR_INVALID_ARG, "eigenvector length differs from the symmetry block size");
    return GAIN_OK;
}

// ------------------------------------------------------------------ plain FP64 path
// The pair's rotational-symmetry table, or NULL (the K-block form).
const WignerTab* wigner_of(gain_engine e, int jindI, int jindF) {
    auto it = e->wigner.find({jindI, jindF});
    return it == e->wigner.end() ? nullptr : it->second.get();
}

// The reference's method for nlo lower levels (device list d_lo) x nup upper levels (d_up) of
// job j's blocks, with the dipole piece now on the device: one half line strength per lower
// state followed by its dot products with every upper vector, into out[nlo][nup].
// kPlainBatch lower states share each launch (and each read of an upper vector); every
// amplitude keeps its own FP64 summation, so it does not depend on the other levels listed.
gain_status plain_amps(gain_engine e, const gain_pair_job* j, int dI, int dF, const int* d_lo, int nlo,
                       const int* d_up, int nup, double* out, int* launches_out) {
    Basis& bI = e->bases[j->jindI];
    Basis& bF = e->bases[j->jindF];
    Inflation& iI = e->infl[j->jindI];
    Inflation& iF = e->infl[j->jindF];
    GammaMaps* mI = gamma_maps(e, j->jindI, j->gammaI, dI);
    GammaMaps* mF = gamma_maps(e, j->jindF, j->gammaF, dF);
    if (!mI || !mF) return GAIN_ERR_OOM;
    PlainLayout& L = e->plain;
    const int key[6] = {j->jindI, j->gammaI, j->jindF, j->gammaF, dI, dF};
    if (!std::equal(key, key + 6, L.key)) {
        L.ctas.clear();
        std::vector<int> flist;
        for (int k = 0; k <= bF.J; ++k) {
            const int s0 = mF->sup_start[k], s1 = mF->sup_start[k + 1];
            for (int b = s0; b < s1; b += kHlsTile) {
                HlsCta c;
                c.kF = k;
                c.f_begin = b;
                c.f_count = std::min(kHlsTile, s1 - b);
                c.pad = 0;
                L.ctas.push_back(c);
            }
        }
        GAIN_TRY(L.d_ctas.upload(L.ctas));
        std::copy(key, key + 6, L.key);
    }
    const Eig& EI = *e->eig[{j->jindI, j->gammaI}];
    const Eig& EF = *e->eig[{j->jindF, j->gammaF}];
    if (EI.ready) GAIN_CUDA(cudaStreamWaitEvent(e->st, EI.ready, 0));
    if (EF.ready) GAIN_CUDA(cudaStreamWaitEvent(e->st, EF.ready, 0));
    const int G = kPlainBatch;
    const int NtF = iF.Ntot[j->gammaF];
    GAIN_TRY(e->primI.alloc((size_t)G * bI.dimen));
    GAIN_TRY(e->hprim.alloc((size_t)G * bF.dimen));
    GAIN_TRY(e->hsym.alloc((size_t)G * NtF));
    cudaStream_t st = e->st;
    int launches = 0;
    for (int l0 = 0; l0 < nlo; l0 += G) {
        const int nb = std::min(G, nlo - l0);
        GAIN_CUDA(launch_expand_levels(iI.dimen, j->gammaI, iI.maxcoeff, dI, iI.sdeg[j->gammaI], iI.Ntot[j->gammaI],
                                       iI.dijterms.p, iI.dicontr.p, iI.dN[j->gammaI]->p, iI.drepres[j->gammaI]->p,
                                       EI.d.p, EI.nsize, d_lo + l0, e->primI.p, bI.dimen, nb, st));
        if (const WignerTab* wt = wigner_of(e, j->jindI, j->jindF)) {
            // rotational-symmetry form (GpuManager::ExecuteRotSymHalfLs): reset, then the dense
            // half line strength of each lower state
            GAIN_CUDA(cudaMemsetAsync(e->hprim.p, 0, sizeof(double) * (size_t)nb * bF.dimen, st));
            for (int b = 0; b < nb; ++b)
                GAIN_CUDA(launch_hls_rotsym(bF.dimen, bI.dimen, wt->nI, wt->nF, wt->maxdeg, bI.dK.p, bF.dK.p, bI.dlev.p,
                                            bF.dlev.p, bI.dvib.p, bF.dvib.p, e->startF, e->endF, e->ncontrF,
                                            e->dipole.p, e->dipN, wt->rot.p, e->primI.p + (size_t)b * bI.dimen,
                                            e->hprim.p + (size_t)b * bF.dimen, st));
            launches += nb;
        } else {
            GAIN_CUDA(launch_hls_needed(L.d_ctas.p, (int)L.ctas.size(), mF->d_support.p, bI.J, bF.J, bI.dtau.p,
                                        bF.dtau.p, bI.dvib.p, bF.dvib.p, mI->d_support.p, mI->d_sup_start.p,
                                        e->startF, e->endF, e->ncontrF, e->dipole.p, e->dipN, e->primI.p, bI.dimen,
                                        e->d3j.p, e->jmax, e->hprim.p, bF.dimen, nb, st));
        }
        GAIN_CUDA(launch_contract(NtF, mF->d_csr_ptr.p, mF->d_csr_col.p, mF->d_csr_val.p, e->hprim.p, bF.dimen,
                                  e->hsym.p, NtF, nb, st));
        GAIN_CUDA(launch_gemv_batch(nup, EF.nsize, EF.d.p, EF.nsize, d_up, e->hsym.p, NtF, nb,
                                    out + (size_t)l0 * nup, nup, st));
        launches += 4;
    }
    if (launches_out) *launches_out = launches;
    return GAIN_OK;
}

gain_status run_plain(gain_engine e, const gain_pair_job* j, int dI, int dF, gain_stats* stats) {
    GAIN_TRY(e->d_lower.upload(j->lower_levels, j->nlower));
    GAIN_TRY(e->d_upper.upload(j->upper_levels, j->nupper));
    GAIN_TRY(e->amp.alloc((size_t)j->nlower * j->nupper));
    cudaStream_t st = e->st;
    GAIN_CUDA(cudaEventRecord(e->ev[0], st));
    int launches = 0;
    GAIN_TRY(plain_amps(e, j, dI, dF, e->d_lower.p, j->nlower, e->d_upper.p, j->nupper, e->amp.p, &launches));
    GAIN_CUDA(cudaEventRecord(e->ev[1], st));
    GAIN_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    GAIN_CUDA(cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]));
    e->amp_rows = j->nlower;
    e->amp_cols = j->nupper;
    e->amp_ld = j->nupper;
    e->have_amp = true;
    e->have_bnd = false;
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->device_ms = ms;
        stats->rows = j->nlower;
        stats->cols = j->nupper;
        stats->kernel_launches = launches;
    }
    return GAIN_OK;
}

gain_status load_piece(gain_engine e, int p);

// The plain path over dipole pieces: one run per piece, amplitudes summed (each piece
// contributes the upper functions of its vibrational range, MultiGpuManager.cpp:240-288).
gain_status run_plain_pieces(gain_engine e, const gain_pair_job* j, int dI, int dF, gain_stats* stats) {
    const size_t n = (size_t)j->nlower * j->nupper;
    double ms = 0;
    long long launches = 0;
    for (int p = 0; p < (int)e->pieces.size(); ++p) {
        GAIN_TRY(load_piece(e, p));
        gain_stats sp;
        GAIN_TRY(run_plain(e, j, dI, dF, &sp));
        ms += sp.device_ms;
        launches += sp.kernel_launches + 1;
        if (p == 0) {
            GAIN_TRY(e->acc.alloc(n));
            GAIN_CUDA(cudaMemcpyAsync(e->acc.p, e->amp.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, e->st));
        } else {
            GAIN_CUDA(launch_add(e->acc.p, e->amp.p, (long)n, e->st));
        }
    }
    GAIN_CUDA(cudaMemcpyAsync(e->amp.p, e->acc.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->device_ms = ms;
        stats->rows = j->nlower;
        stats->cols = j->nupper;
        stats->kernel_launches = launches;
    }
    return GAIN_OK;
}

// ------------------------------------------------------------------ split path
struct SplitParams {
    int beta, slices, chunks;
};

// Digits and chunking from the inner length K of the exact accumulations: the Cauchy-Schwarz
// certificate needs ||d_i|| ||d_j|| < 2^24 over every chunk.  Balanced residual digits have
// ||d||^2 ~ K_chunk 4^beta / 12, and over a chunk of a few thousand digits the norms of
// eigenvector-like rows stay within a few percent of it, so K_chunk 4^beta / 12 <=
// 2^24 / kChunkMargin.  An output whose digit norms exceed the budget anyway fails its
// certificate and is recomputed in FP64.  (A factor-two margin took 8 chunks at K = 12 288
// and 8-bit digits, this one 5: 168 -> 105 accumulator drains per output tile.)
// Without an explicit digit width the widest one (from beta_default down) whose chunks fit
// MAX_CHUNKS is taken: wider digits mean fewer digit products for the same bits.
constexpr double kChunkMargin = 1.25;
SplitParams choose_params(int K, const gain_split_opts* o, int bits, int beta_default) {
    auto chunks_for = [K](int beta) {
        const double limit = 16777216.0 / kChunkMargin * 12.0 / std::ldexp(1.0, 2 * beta);
        return std::max(1, (int)std::ceil((double)K / limit));
    };
    SplitParams p;
    p.beta = (o && o->beta) ? o->beta : beta_default;
    if (!(o && (o->beta || o->kchunks)))
        while (p.beta > 4 && chunks_for(p.beta) > split::MAX_CHUNKS) --p.beta;
    p.slices = (o && o->slices) ? o->slices : (bits + p.beta - 1) / p.beta;
    p.chunks = (o && o->kchunks) ? o->kchunks : chunks_for(p.beta);
    p.chunks = std::min(p.chunks, split::MAX_CHUNKS);
    return p;
}

// Bound of the int64 fixed-point recombination, units of 2^{eA+eB}: each digit product adds
// at most one truncated unit of 2^{-kFixTotal}; the final int64 -> double conversion adds a
// relative 2^-53, negligible against tol, absorbed by the 1.01.
float fix_const(int nprods) {
    return (float)((double)nprods * std::ldexp(1.0, -split::kFixTotal) * 1.01);
}

// Digit products of a tile in chunk-major order, then by A digit plane: while the persistent
// CTAs work through one inner chunk, that chunk's digit tiles for all their rows and columns
// (tens of MB) stay in L2 and are read from HBM once, and consecutive passes reuse the same
// A plane (product-major order re-streamed every plane of every chunk from HBM).  The int64
// recombination does not depend on the order.
std::vector<split::Prod> make_prods(const SplitParams& p, int fuse = 1) {
    std::vector<split::Prod> v;
    auto add = [&](int i, int j, int c, bool open, bool close) {
        split::Prod q;
        memset(&q, 0, sizeof q);
        q.ia = i;
        q.ib = j;
        q.t = i + j;
        q.chunk = c;
        q.open = open ? 1 : 0;
        q.close = close ? 1 : 0;
        v.push_back(q);
    };
    if (fuse <= 1) {
        for (int c = 0; c < p.chunks; ++c)
            for (int i = 0; i < p.slices; ++i)
                for (int j = 0; i + j < p.slices; ++j) add(i, j, c, true, true);
        return v;
    }
    // fused: per chunk and weight t, the t + 1 products (i, t - i) in groups of at most `fuse`
    // that share one accumulator
    for (int c = 0; c < p.chunks; ++c)
        for (int t = 0; t < p.slices; ++t)
            for (int i = 0; i <= t; ++i) {
                const int k = i % fuse;
                add(i, t - i, c, k == 0, k == fuse - 1 || i == t);
            }
    return v;
}

// Tile order for L2 reuse: a list built column-block-major (all row tiles of a column block,
// then the next column block) is regrouped into row groups of kRowGroup row tiles: for each
// group, every column block's tiles of those rows.  The persistent CTAs take consecutive
// tiles, so the concurrent tiles then share kRowGroup A row tiles and about units/kRowGroup
// B column tiles, whose digits stay in L2 across the digit products (with all row tiles of a
// tall operand per column block, the A tiles of one product exceed L2 and are read from DRAM
// again for every product).  key_split (optional) keeps tiles with key_split(t) = 0 before the
// others (the upper halves of a run whose upper vectors are still arriving).
constexpr int kRowGroup = 8;
template <class Split>
void row_grouped(std::vector<split::Tile>& t, int mstep, Split key_split) {
    std::stable_sort(t.begin(), t.end(), [&](const split::Tile& a, const split::Tile& b) {
        const int sa = key_split(a), sb = key_split(b);
        if (sa != sb) return sa < sb;
        return a.m0 / (kRowGroup * mstep) < b.m0 / (kRowGroup * mstep);
    });
}
void row_grouped(std::vector<split::Tile>& t, int mstep) {
    row_grouped(t, mstep, [](const split::Tile&) { return 0; });
}

// Spread of tiles over `units` persistent CTAs (CTA pairs) in list order: each tile goes to
// the unit that frees up first, the order a dynamic scheduler would give, so that the tiles
// running at any moment are neighbours in the list and share their operands' digits in L2 as
// in a single run (a longest-first spread scatters every unit's k-th tile over the whole
// list, and the digits of each then come from DRAM).  The jobs (tile groups) with the
// costliest tiles go first, so that cheap tiles even out the end.  The list is laid out so
// that unit u runs entries u, u + units, ... (empty slots: group -1).
std::vector<split::Tile> list_schedule(const std::vector<split::Tile>& tiles, const std::vector<double>& cost,
                                       int units) {
    std::map<int, double> job_cost;
    for (size_t i = 0; i < tiles.size(); ++i) job_cost[tiles[i].group] = std::max(job_cost[tiles[i].group], cost[i]);
    std::vector<int> order(tiles.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return job_cost[tiles[a].group] > job_cost[tiles[b].group]; });
    std::vector<std::vector<int>> per(units);
    typedef std::pair<double, int> LU;
    std::priority_queue<LU, std::vector<LU>, std::greater<LU>> heap;
    for (int u = 0; u < units; ++u) heap.push({0.0, u});
    for (int t : order) {
        LU top = heap.top();
        heap.pop();
        per[top.second].push_back(t);
        top.first += cost[t];
        heap.push(top);
    }
    size_t depth = 0;
    for (auto& v : per) depth = std::max(depth, v.size());
    split::Tile empty;
    memset(&empty, 0, sizeof empty);
    empty.group = -1;
    std::vector<split::Tile> out(depth * units, empty);
    for (int u = 0; u < units; ++u)
        for (size_t k = 0; k < per[u].size(); ++k) out[k * units + u] = tiles[per[u][k]];
    return out;
}

// Products fused per accumulator in the first GEMM: only where each product is short (fewer
// than 16 k-blocks per tile, so that draining the accumulator after every product would pace
// the tensor pipe); as many as keep the expected sum of their digit norms' products, K_chunk
// 4^beta / 12 each for balanced digits, within 2^23 (a factor-two margin: the first GEMM's
// band rows are short and sparse, so their norms vary more than an eigenvector row's).
// The exactness certificate checks it per output.  GAINLS_FUSE1=0 disables.
int gemm1_fuse(const PairLayout& L, const SplitParams& p1) {
    if (const char* f = getenv("GAINLS_FUSE1"))
        if (f[0] == '0') return 1;
    const int kchunk = L.W / std::max(1, p1.chunks);
    if (kchunk / split::BK >= 16) return 1;
    const double per = (double)kchunk * std::ldexp(1.0, 2 * p1.beta) / 12.0;
    const int f = (int)std::floor(8388608.0 / std::max(per, 1.0));
    return std::max(1, std::min(p1.slices, f));
}

gain_status launch_layout_band(gain_engine e, const gain_pair_job* j);

gain_status build_layout(gain_engine e, const gain_pair_job* j, int dI, int dF, GammaMaps* mI, GammaMaps* mF) {
    const int key[6] = {j->jindI, j->gammaI, j->jindF, j->gammaF, dI, dF};
    const std::array<int, 6> akey = {key[0], key[1], key[2], key[3], key[4], key[5]};
    auto it = e->layouts.find(akey);
    if (it == e->layouts.end()) {
        // bound the cache: band and band digits of every cached pair below a quarter of the
        // device memory that is free now (the current pair's are built next)
        size_t cached = 0;
        for (auto& kv : e->layouts) cached += layout_bytes(*kv.second);
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && cached > free_b / 4) {
            GAIN_CUDA(cudaStreamSynchronize(e->st));
            e->layouts.clear();
        }
        it = e->layouts.emplace(akey, std::make_shared<PairLayout>()).first;
    }
    e->cur = it->second.get();
    PairLayout& L = *e->cur;
    const WignerTab* wt = wigner_of(e, j->jindI, j->jindF);
    const long wv = wt ? wt->version : 0;
    if (std::equal(key, key + 6, L.key) && L.dip_version == e->dip_version && L.wig_version == wv) return GAIN_OK;
    L.rotsym = wt != nullptr;
    Basis& bI = e->bases[j->jindI];
    Basis& bF = e->bases[j->jindF];
    // The units of each layout: with selection expansions the symmetric functions (a primitive
    // times a coefficient each); otherwise the primitives the expansions touch, the lower
    // vectors expanded before the first GEMM and H contracted after it.
    // With mixing expansions whose symmetric functions each combine primitives of one K, the
    // band is formed over symmetric functions directly (symband); otherwise GEMM1 runs over
    // primitives (general).
    auto one_k = [](const GammaMaps* m, const Basis& b, std::vector<int>& first) {
        const int n = (int)m->csr_ptr.size() - 1;
        first.assign(n, 0);
        for (int sy = 0; sy < n; ++sy) {
            const int q0 = m->csr_ptr[sy], q1 = m->csr_ptr[sy + 1];
            if (q0 == q1) continue;
            first[sy] = m->csr_col[q0];
            for (int q = q0; q < q1; ++q)
                if (b.K[m->csr_col[q]] != b.K[first[sy]]) return false;
        }
        return true;
    };
    std::vector<int> firstI, firstF;
    const bool sel = mI->selection && mF->selection;
    // GAINLS_SPLIT_FORM=primitive keeps GEMM1 over primitives for every mixing expansion
    const char* form_env = getenv("GAINLS_SPLIT_FORM");
    const bool force_prim = form_env && std::string(form_env) == "primitive";
    L.symband = !sel && !force_prim && one_k(mI, bI, firstI) && one_k(mF, bF, firstF);
    L.general = !sel && !L.symband;
    const std::vector<int>& uI = L.general ? mI->support : (L.symband ? firstI : mI->sym_prim);
    const std::vector<int>& uF = L.general ? mF->support : (L.symband ? firstF : mF->sym_prim);
    auto coefI = [&](int s) { return sel ? mI->sym_coef[s] : 1.0; };
    auto coefF = [&](int s) { return sel ? mF->sym_coef[s] : 1.0; };
    L.nI = (int)uI.size();
    L.nF = (int)uF.size();
    // lower layout: units grouped by K, each group padded to BK
    std::vector<std::vector<int>> byK(bI.J + 1);
    for (int s = 0; s < L.nI; ++s) byK[bI.K[uI[s]]].push_back(s);
    L.kpad_startI.assign(bI.J + 2, 0);
    for (int k = 0; k <= bI.J; ++k) L.kpad_startI[k + 1] = L.kpad_startI[k] + round_up((int)byK[k].size(), split::BK);
    L.kpadI = std::max(L.kpad_startI[bI.J + 1], split::BK);
    L.colposI.assign(L.nI, 0);
    L.i_sym.assign(L.kpadI, -1);
    L.i_prim.assign(L.kpadI, -1);
    L.i_coef.assign(L.kpadI, 0.0);
    for (int k = 0; k <= bI.J; ++k)
        for (size_t x = 0; x < byK[k].size(); ++x) {
            const int s = byK[k][x], pos = L.kpad_startI[k] + (int)x;
            L.colposI[s] = pos;
            L.i_sym[pos] = L.general ? uI[s] : s;   // source column: primitive (expanded) or symmetric
            L.i_prim[pos] = uI[s];
            L.i_coef[pos] = coefI(s);
        }
    // upper layout: grouped by K, each group padded to BN
    std::vector<std::vector<int>> byKF(bF.J + 1);
    for (int s = 0; s < L.nF; ++s) byKF[bF.K[uF[s]]].push_back(s);
    L.fblocks.clear();
    int pos = 0;
    L.colposF.assign(L.nF, 0);
    std::vector<int> f_k;
    for (int k = 0; k <= bF.J; ++k) {
        const int n = (int)byKF[k].size();
        if (!n) continue;
        const int np = round_up(n, split::BN);
        L.fblocks.push_back({pos, pos + np});
        for (int x = 0; x < np; ++x) f_k.push_back(k);
        pos += np;
    }
    L.fpad = std::max(pos, split::BN);
    if (f_k.empty()) f_k.assign(L.fpad, 0);
    L.f_sym.assign(L.fpad, -1);
    L.f_prim.assign(L.fpad, -1);
    L.f_coef.assign(L.fpad, 0.0);
    L.band_k0.assign(L.fpad, 0);
    L.band_len.assign(L.fpad, 0);
    {
        int p2 = 0;
        for (int k = 0; k <= bF.J; ++k) {
            const int n = (int)byKF[k].size();
            if (!n) continue;
            for (int x = 0; x < n; ++x) {
                const int s = byKF[k][x];
                L.colposF[s] = p2 + x;
                L.f_sym[p2 + x] = s;
                L.f_prim[p2 + x] = uF[s];
                L.f_coef[p2 + x] = coefF(s);
            }
            p2 += round_up(n, split::BN);
        }
    }
    L.W = split::BK;
    for (int r = 0; r < L.fpad; ++r) {
        if (L.rotsym) {   // no K sparsity: every upper row spans the whole lower layout
            L.band_k0[r] = 0;
            L.band_len[r] = L.kpadI;
            L.W = L.kpadI;
            continue;
        }
        const int kF = f_k[r];
        const int klo = std::max(kF - 1, 0), khi = std::min(kF + 1, bI.J);
        if (klo > khi) continue;
        L.band_k0[r] = L.kpad_startI[klo];
        L.band_len[r] = L.kpad_startI[khi + 1] - L.kpad_startI[klo];
        L.W = std::max(L.W, L.band_len[r]);
    }
    if (L.symband) {   // each padded row / column: the primitives of its symmetric function
        auto build = [](const GammaMaps* m, const std::vector<int>& unit_at, std::vector<int>& ptr,
                        std::vector<int>& col, std::vector<double>& val) {
            ptr.assign(unit_at.size() + 1, 0);
            col.clear();
            val.clear();
            for (size_t x = 0; x < unit_at.size(); ++x) {
                const int sy = unit_at[x];
                if (sy >= 0)
                    for (int q = m->csr_ptr[sy]; q < m->csr_ptr[sy + 1]; ++q) {
                        col.push_back(m->csr_col[q]);
                        val.push_back(m->csr_val[q]);
                    }
                ptr[x + 1] = (int)col.size();
            }
        };
        build(mI, L.i_sym, L.ic_ptr, L.ic_col, L.ic_val);
        build(mF, L.f_sym, L.fr_ptr, L.fr_col, L.fr_val);
        if (L.ic_col.empty()) { L.ic_col.push_back(0); L.ic_val.push_back(0.0); }
        if (L.fr_col.empty()) { L.fr_col.push_back(0); L.fr_val.push_back(0.0); }
        GAIN_TRY(L.d_ic_ptr.upload(L.ic_ptr));
        GAIN_TRY(L.d_ic_col.upload(L.ic_col));
        GAIN_TRY(L.d_ic_val.upload(L.ic_val));
        GAIN_TRY(L.d_fr_ptr.upload(L.fr_ptr));
        GAIN_TRY(L.d_fr_col.upload(L.fr_col));
        GAIN_TRY(L.d_fr_val.upload(L.fr_val));
    }
    if (L.general) {
        // T_F^T as CSR over the symmetric functions, its columns moved to the F layout
        Inflation& iF = e->infl[j->jindF];
        L.nsymF = iF.Ntot[j->gammaF];
        L.ntpad = std::max(round_up(L.nsymF, split::BK), split::BK);
        std::vector<int> unit_of(bF.dimen, -1);
        for (int u = 0; u < L.nF; ++u) unit_of[uF[u]] = u;
        L.cF_ptr.assign(mF->csr_ptr.begin(), mF->csr_ptr.end());
        L.cF_col.resize(mF->csr_col.size());
        L.cF_val.assign(mF->csr_val.begin(), mF->csr_val.end());
        std::vector<double> rowsum(L.nF, 0.0);
        double colmax = 0.0;
        int kmax = 1;
        for (int sy = 0; sy < L.nsymF; ++sy) {
            double cs = 0.0;
            kmax = std::max(kmax, L.cF_ptr[sy + 1] - L.cF_ptr[sy]);
            for (int q = L.cF_ptr[sy]; q < L.cF_ptr[sy + 1]; ++q) {
                const int u = unit_of[mF->csr_col[q]];
                L.cF_col[q] = L.colposF[u];
                cs += std::fabs(L.cF_val[q]);
                rowsum[u] += std::fabs(L.cF_val[q]);
            }
            colmax = std::max(colmax, cs);
        }
        double rowmax = 0.0;
        for (double v : rowsum) rowmax = std::max(rowmax, v);
        // Schur bound of ||T_F||_2, and the FP64 summation bound gamma_k = k u / (1 - k u)
        L.sigmaF = std::sqrt(rowmax * colmax) * (1.0 + 1e-12);
        const double u = std::ldexp(1.0, -53);
        L.gamF = (kmax * u) / (1.0 - kmax * u) * (1.0 + 1e-12);
        std::vector<int> ident(L.nsymF);
        for (int q = 0; q < L.nsymF; ++q) ident[q] = q;
        GAIN_TRY(L.d_cF_ptr.upload(L.cF_ptr));
        GAIN_TRY(L.d_cF_col.upload(L.cF_col));
        GAIN_TRY(L.d_cF_val.upload(L.cF_val));
        GAIN_TRY(L.d_ident.upload(ident));
    }
    GAIN_TRY(L.d_colposI.upload(L.colposI));
    GAIN_TRY(L.d_i_sym.upload(L.i_sym));
    GAIN_TRY(L.d_i_prim.upload(L.i_prim));
    GAIN_TRY(L.d_i_coef.upload(L.i_coef));
    GAIN_TRY(L.d_colposF.upload(L.colposF));
    GAIN_TRY(L.d_f_sym.upload(L.f_sym));
    GAIN_TRY(L.d_f_prim.upload(L.f_prim));
    GAIN_TRY(L.d_f_coef.upload(L.f_coef));
    GAIN_TRY(L.d_band_k0.upload(L.band_k0));
    GAIN_TRY(L.d_band_len.upload(L.band_len));
    GAIN_TRY(L.band.alloc((size_t)L.fpad * L.W));
    GAIN_TRY(launch_layout_band(e, j));
    L.beta1 = 0;
    L.s1 = 0;
    L.c1 = 0;
    std::copy(key, key + 6, L.key);
    L.dip_version = e->dip_version;
    L.wig_version = wv;
    return GAIN_OK;
}

// The rotational-dipole band of the current layout from the dipole piece now on the device
// (rows whose upper vibrational index lies outside the piece are zero).
gain_status launch_layout_band(gain_engine e, const gain_pair_job* j) {
    PairLayout& L = *e->cur;
    const WignerTab* wt = wigner_of(e, j->jindI, j->jindF);
    Basis& bI = e->bases[j->jindI];
    Basis& bF = e->bases[j->jindF];
    split::BandArgs ba;
    ba.fpad = L.fpad;
    ba.W = L.W;
    ba.f_prim = L.d_f_prim.p;
    ba.f_coef = L.d_f_coef.p;
    ba.band_k0 = L.d_band_k0.p;
    ba.kpadI = L.kpadI;
    ba.i_prim = L.d_i_prim.p;
    ba.i_coef = L.d_i_coef.p;
    ba.KI = bI.dK.p;
    ba.tauI = bI.dtau.p;
    ba.vibI = bI.dvib.p;
    ba.KF = bF.dK.p;
    ba.tauF = bF.dtau.p;
    ba.vibF = bF.dvib.p;
    ba.jI = bI.J;
    ba.jF = bF.J;
    ba.jmax = e->jmax;
    ba.threej = e->d3j.p;
    ba.dipole = e->dipole.p;
    ba.dipN = e->dipN;
    ba.startF = e->startF;
    ba.endF = e->endF;
    ba.ncontrF = e->ncontrF;
    ba.band = L.band.p;
    ba.wigner = wt ? wt->rot.p : nullptr;
    if (wt) {   // the rotsym form reads level indices where the K-block form reads tau parities
        ba.tauI = bI.dlev.p;
        ba.tauF = bF.dlev.p;
    }
    ba.nlevelI = wt ? wt->nI : 0;
    ba.nlevelF = wt ? wt->nF : 0;
    ba.maxdeg = wt ? wt->maxdeg : 0;
    ba.f_ptr = L.symband ? L.d_fr_ptr.p : nullptr;
    ba.f_col = L.symband ? L.d_fr_col.p : nullptr;
    ba.f_val = L.symband ? L.d_fr_val.p : nullptr;
    ba.i_ptr = L.symband ? L.d_ic_ptr.p : nullptr;
    ba.i_col = L.symband ? L.d_ic_col.p : nullptr;
    ba.i_val = L.symband ? L.d_ic_val.p : nullptr;
    GAIN_CUDA(split::launch_band(ba, e->st));
    ++e->launches;
    return GAIN_OK;
}

// Copy dipole piece p of the host list into the device buffer (after the work queued on the
// engine's stream that reads the previous piece).
gain_status load_piece(gain_engine e, int p) {
    if (e->piece_loaded == p) return GAIN_OK;
    const auto& hp = e->pieces[p];
    const size_t n = (size_t)3 * e->dipN * (hp.endF - hp.startF);
    size_t mx = 0;
    for (auto& q : e->pieces) mx = std::max(mx, (size_t)3 * e->dipN * (q.endF - q.startF));
    GAIN_TRY(e->dipole.alloc(mx));
    GAIN_CUDA(cudaMemcpyAsync(e->dipole.p, hp.host, sizeof(double) * n, cudaMemcpyHostToDevice, e->st));
    e->startF = hp.startF;
    e->endF = hp.endF;
    e->ncontrF = hp.endF - hp.startF;
    e->piece_loaded = p;
    ++e->dip_version;
    return GAIN_OK;
}

// Digits of nrows source rows into dig [slices][rows_pad][kpad].  host_map (the host copy of
// col_map, increasing; NULL for the identity) locates each GEMM chunk's source columns.
split::SliceArgs slice_args(const double* src, long ld, const int* src_rows, int nrows, int ncols,
                            const int* col_map, const std::vector<int>* host_map, int kpad, int rows_pad,
                            __nv_bfloat16* dig, const SplitParams& p, StatsDev& stv, bool with_inerr,
                            const float* inerr_prev, const int* e_prev, const int* col_inv = nullptr,
                            int grid_limit = 0, int row0 = 0) {
    // row0: the output rows start at row row0 of the digit and statistics arrays
    split::SliceArgs a;
    memset(&a, 0, sizeof a);
    a.grid_limit = grid_limit;
    a.col_inv = col_inv;
    const int nkb = kpad / split::BK;
    for (int c = 0; c <= p.chunks; ++c) {
        const int dest0 = c == p.chunks ? kpad : (int)(((long)c * nkb) / p.chunks) * split::BK;
        int s0;
        if (c == p.chunks) s0 = ncols;
        else if (!host_map) s0 = std::min(dest0, ncols);
        else s0 = (int)(std::lower_bound(host_map->begin(), host_map->begin() + ncols, dest0) - host_map->begin());
        a.src_chunk[c] = s0;
    }
    a.src = src;
    a.ld_src = ld;
    a.src_rows = src_rows;
    a.nrows = nrows;
    a.ncols = ncols;
    a.col_map = col_map;
    a.kpad = kpad;
    a.slice_stride = (long)rows_pad * kpad;
    a.digits = dig + (size_t)row0 * kpad;
    a.slices = p.slices;
    a.beta = p.beta;
    a.nchunks = p.chunks;
    a.st = stv.view(with_inerr, (size_t)row0, p.chunks);
    a.inerr2_prev = inerr_prev ? inerr_prev + row0 : nullptr;
    a.e_prev = e_prev ? e_prev + row0 : nullptr;
    return a;
}

gain_status slice(gain_engine e, const double* src, long ld, const int* src_rows, int nrows, int ncols,
                  const int* col_map, const std::vector<int>* host_map, int kpad, int rows_pad,
                  __nv_bfloat16* dig, const SplitParams& p, StatsDev& stv, bool with_inerr,
                  const float* inerr_prev, const int* e_prev, cudaStream_t st, const int* col_inv = nullptr,
                  int grid_limit = 0, int row0 = 0) {
    const split::SliceArgs a = slice_args(src, ld, src_rows, nrows, ncols, col_map, host_map, kpad, rows_pad, dig, p,
                                          stv, with_inerr, inerr_prev, e_prev, col_inv, grid_limit, row0);
    GAIN_CUDA(split::launch_slice(a, st));
    ++e->launches;
    return GAIN_OK;
}

// The band digits of layout L for the first GEMM's digit configuration p1 (kept until the
// configuration or the band changes) and their tensor maps.
gain_status layout_band_digits(gain_engine e, PairLayout& L, const SplitParams& p1, cudaStream_t st) {
    if (L.beta1 != p1.beta || L.s1 != p1.slices || L.c1 != p1.chunks) {
        GAIN_TRY(L.bandDig.alloc((size_t)p1.slices * L.fpad * L.W));
        GAIN_TRY(L.bandDig.zero(st, (size_t)p1.slices * L.fpad * L.W));
        GAIN_TRY(L.bandStats.alloc(L.fpad, p1.chunks, false));
        GAIN_TRY(L.bandStats.zero(st, L.fpad, p1.chunks, false));
        GAIN_TRY(slice(e, L.band.p, L.W, nullptr, L.fpad, L.W, nullptr, nullptr, L.W, L.fpad, L.bandDig.p, p1,
                       L.bandStats, false, nullptr, nullptr, st));
        if (!split::make_digit_map(&L.tmBand, L.bandDig.p, L.W, L.fpad, p1.slices) ||
            !split::make_digit_map(&L.tmBandPair, L.bandDig.p, L.W, L.fpad, p1.slices, split::BN / 2))
            return set_error(GAIN_ERR_CUDA, "cuTensorMapEncodeTiled failed for the band digits");
        L.beta1 = p1.beta;
        L.s1 = p1.slices;
        L.c1 = p1.chunks;
    }
    return GAIN_OK;
}

// Digit configuration of the first GEMM for layout L: 53 - log2(W + 64) + 6 bits between 46
// and 56 (every H entry must stay within the FP64 bound of its dot product, which loosens
// with the band width W); one inner chunk per band tile with the digits narrowed until it
// stays exact, or (rotational-symmetry form, every tile spanning the whole lower layout)
// chunks as in the second GEMM.  GAINLS_GEMM1_BITS (40..62) overrides the bits.
SplitParams gemm1_params(const PairLayout& L, const gain_split_opts* opts) {
    gain_split_opts o1{};
    if (opts) o1.beta = opts->beta;
    int bits1 = (int)std::ceil(53.0 - std::log2((double)L.W + 64.0) + 6.0);
    bits1 = std::max(46, std::min(56, bits1));
    if (const char* b1 = getenv("GAINLS_GEMM1_BITS")) bits1 = std::max(40, std::min(62, atoi(b1)));
    SplitParams p1x;
    if (L.rotsym) {
        p1x = choose_params(L.W, &o1, bits1, 8);
    } else {
        p1x = choose_params(L.W, &o1, bits1, 7);
        p1x.chunks = 1;
        while (p1x.beta > 4 && (double)L.W * std::ldexp(1.0, 2 * p1x.beta) / 12.0 > 8388608.0) {
            --p1x.beta;
            p1x.slices = (bits1 + p1x.beta - 1) / p1x.beta;
        }
    }
    return p1x;
}

bool digits_supported(const SplitParams& p1, const SplitParams& p2) {
    return !(p1.slices * p1.beta > 62 || p2.slices * p2.beta > 62 || p1.slices > split::MAX_SLICES ||
             p2.slices > split::MAX_SLICES || p1.beta < 2 || p1.beta > 8 || p2.beta < 2 || p2.beta > 8 ||
             2 * (p2.slices - 1) * p2.beta > 126 || 2 * (p1.slices - 1) * p1.beta > 126);
}

gain_status run_split(gain_engine e, const gain_pair_job* j, int dI, int dF, const gain_split_opts* opts,
                      gain_stats* stats) {
    GammaMaps* mI = gamma_maps(e, j->jindI, j->gammaI, dI);
    GammaMaps* mF = gamma_maps(e, j->jindF, j->gammaF, dF);
    if (!mI || !mF) return GAIN_ERR_OOM;
    const double tol = (opts && opts->tol > 0) ? opts->tol : 4.5e-9;
    cudaStream_t st = e->st;
    const long launches0 = e->launches;
    GAIN_CUDA(cudaEventRecord(e->ev[0], st));
    // dipole pieces (MultiGpuManager::ExecuteHalfLs's block loop): H accumulates the first
    // GEMM of every piece, the second GEMM runs once
    const int npieces = e->pieces.size() > 1 ? (int)e->pieces.size() : 1;
    if (npieces > 1) GAIN_TRY(load_piece(e, 0));
    GAIN_TRY(build_layout(e, j, dI, dF, mI, mF));
    PairLayout& L = *e->cur;
    const Eig& EI = *e->eig[{j->jindI, j->gammaI}];
    const Eig& EF = *e->eig[{j->jindF, j->gammaF}];
    // an asynchronous upload of the lower vectors must land before the lower slicing; the upper
    // vectors are awaited on the second stream only, so their copy overlaps the lower side
    if (EI.ready) GAIN_CUDA(cudaStreamWaitEvent(st, EI.ready, 0));

    // First GEMM: about 49 bits at band widths near 3000 (its error reaches every amplitude
    // through ||dH||_2 ||u||_2; every entry must certify FP64-grade), see gemm1_params.
    // Second GEMM: 48 bits (8-bit digits in up to MAX_CHUNKS chunks, else 7 x 7 bits);
    // options (beta, slices, kchunks) apply to it.
    const SplitParams p1x = gemm1_params(L, opts);
    const int K2 = L.general ? L.ntpad : L.fpad;   // inner dimension of the second GEMM
    const SplitParams p2 = choose_params(K2, opts, 48, 8);
    if (!digits_supported(p1x, p2)) return set_error(GAIN_ERR_INVALID_ARG, "unsupported digit configuration");

    // band digits (cached per digit configuration)
    auto band_digits = [&]() -> gain_status { return layout_band_digits(e, L, p1x, st); };
    GAIN_TRY(band_digits());

    // CTA pairs (256 x 128 tiles) whenever the lower states fill more than one 128-row block;
    // GAINLS_GEMM_PAIR=0 keeps single-CTA tiles
    const int B = j->nlower;
    const char* pair_env = getenv("GAINLS_GEMM_PAIR");
    const bool pair = B > split::BM && !(pair_env && pair_env[0] == '0');
    const int mstep = pair ? 2 * split::BM : split::BM;
    const int Bpad = round_up(B, mstep);
    const int Nu = j->nupper, Nupad = round_up(Nu, split::BN);
    // While the upper vectors are still arriving in two parts, the upper side runs in two
    // halves: the first half's digits and amplitude GEMM start when the first part lands.
    int Nu2 = 0;
    bool arriving = false;
    if (EF.ready && EF.ready_head && EF.head_rows > 0 && Nu >= 2 * split::BN) {
        const cudaError_t q = cudaEventQuery(EF.ready);
        if (q == cudaErrorNotReady) (void)cudaGetLastError();   // not an error: the copy is in flight
        const char* halves = getenv("GAINLS_UPPER_HALVES");     // "force": also after the copy landed
        arriving = q == cudaErrorNotReady || (halves && std::string(halves) == "force");
    }
    if (arriving) {
        const int cand = (Nupad / split::BN + 1) / 2 * split::BN;   // the upper blocks halved, rounded up
        bool in_head = true;
        for (int u = 0; u < cand && in_head; ++u) in_head = j->upper_levels[u] < EF.head_rows;
        if (in_head) Nu2 = cand;
    }
    // Small uploads stay synchronous: an asynchronous copy on this stream would queue in the
    // host-to-device engine behind an eigenvector copy still in flight and hold GEMM 1 back.
    GAIN_TRY(e->d_lower.upload(j->lower_levels, B));
    GAIN_TRY(e->d_upper.upload(j->upper_levels, Nu));
    GAIN_TRY(e->counters.alloc(4));
    GAIN_TRY(e->counters.zero(st, 4));
    GAIN_TRY(e->ull.alloc(4));
    GAIN_TRY(e->ull.zero(st, 4));
    GAIN_TRY(e->err.alloc(1));
    GAIN_TRY(e->err.zero(st, 1));
    GAIN_TRY(e->flags1.alloc(kMaxFlags));
    GAIN_TRY(e->flags2.alloc(kMaxFlags));
    // capacity of the refinement lists (GAINLS_MAX_FLAGS lowers it, to exercise the overflow
    // handling on small cases)
    int max_flags = kMaxFlags;
    if (const char* mf = getenv("GAINLS_MAX_FLAGS")) max_flags = std::max(0, std::min(kMaxFlags, atoi(mf)));

    // Digit buffers and their row statistics are cleared only when their shape or layout
    // changes: padding rows and columns are never written, every other entry is.
    const long lkey = (long)L.key[0] * 1000003L + L.key[1] * 1009L + L.key[2] * 31L + L.key[3];
    const size_t vdig = (size_t)p1x.slices * Bpad * L.kpadI;
    const size_t hdig = (size_t)p2.slices * Bpad * K2;
    const size_t udig = (size_t)p2.slices * Nupad * K2;
    GAIN_TRY(e->Vdig.alloc(vdig));
    GAIN_TRY(e->Vst.alloc(Bpad, p1x.chunks, false));
    GAIN_TRY(e->Hdig.alloc(hdig));
    GAIN_TRY(e->Hst.alloc(Bpad, p2.chunks, true));
    GAIN_TRY(e->Udig.alloc(udig));
    GAIN_TRY(e->Ust.alloc(Nupad, p2.chunks, false));
    const std::vector<long> kV = {lkey, p1x.slices, p1x.beta, p1x.chunks, B, Bpad, (long)(uintptr_t)e->Vdig.p};
    const std::vector<long> kH = {lkey, p2.slices, p2.chunks, B, Bpad, (long)(uintptr_t)e->Hdig.p};
    const std::vector<long> kU = {lkey, p2.slices, p2.chunks, Nu, Nupad, (long)(uintptr_t)e->Udig.p};
    if (e->zkey_V != kV) {
        GAIN_TRY(e->Vdig.zero(st, vdig));
        GAIN_TRY(e->Vst.zero(st, Bpad, p1x.chunks, false));
        e->zkey_V = kV;
    }
    if (e->zkey_H != kH) {
        GAIN_TRY(e->Hdig.zero(st, hdig));
        GAIN_TRY(e->Hst.zero(st, Bpad, p2.chunks, true));
        e->zkey_H = kH;
    }
    if (e->zkey_U != kU) {
        GAIN_TRY(e->Udig.zero(st, udig));
        GAIN_TRY(e->Ust.zero(st, Nupad, p2.chunks, false));
        e->zkey_U = kU;
    }

    // The upper slicing runs on the second stream from here on.  It cannot share SMs with the
    // first GEMM (the GEMM's 256-register warps fill two SM sub-partitions' register files),
    // so it overlaps the lower slicing and precedes the GEMM.
    GAIN_CUDA(cudaEventRecord(e->ev[6], st));

    // ---- lower vectors -> digits in the padded lower layout (expanded to primitives first
    // when the expansion mixes them)
    const Basis& bIs = e->bases[j->jindI];
    if (L.general && B > 65535)
        return set_error(GAIN_ERR_UNSUPPORTED, "split path with a mixing expansion: at most 65535 lower states per run");
    if (L.general) {
        Inflation& iI = e->infl[j->jindI];
        GAIN_TRY(e->primI.alloc((size_t)B * bIs.dimen));
        GAIN_TRY(e->iota.alloc(B));
        {
            std::vector<int> io(B);
            for (int b = 0; b < B; ++b) io[b] = b;
            GAIN_CUDA(cudaMemcpyAsync(e->iota.p, io.data(), sizeof(int) * B, cudaMemcpyHostToDevice, st));
            GAIN_CUDA(cudaStreamSynchronize(st));
        }
        for (int b0 = 0; b0 < B; b0 += 65535) {
            const int nb = std::min(65535, B - b0);
            GAIN_CUDA(launch_expand_levels(iI.dimen, j->gammaI, iI.maxcoeff, dI, iI.sdeg[j->gammaI], iI.Ntot[j->gammaI],
                                           iI.dijterms.p, iI.dicontr.p, iI.dN[j->gammaI]->p, iI.drepres[j->gammaI]->p,
                                           EI.d.p, EI.nsize, e->d_lower.p + b0, e->primI.p + (size_t)b0 * bIs.dimen,
                                           bIs.dimen, nb, st));
            ++e->launches;
        }
        GAIN_TRY(slice(e, e->primI.p, bIs.dimen, nullptr, B, bIs.dimen, nullptr, nullptr, L.kpadI, Bpad, e->Vdig.p,
                       p1x, e->Vst, false, nullptr, nullptr, st, L.d_i_sym.p));
    } else {
        GAIN_TRY(slice(e, EI.d.p, EI.nsize, e->d_lower.p, B, EI.nsize, L.d_colposI.p, &L.colposI, L.kpadI, Bpad,
                       e->Vdig.p, p1x, e->Vst, false, nullptr, nullptr, st, L.d_i_sym.p));
    }
    CUtensorMap tmV, tmH, tmU;
    if (!split::make_digit_map(&tmV, e->Vdig.p, L.kpadI, Bpad, p1x.slices))
        return set_error(GAIN_ERR_CUDA, "cuTensorMapEncodeTiled failed (lower digits)");

    // ---- GEMM 1: H = V M (one pass per dipole piece)
    const int fuse1 = gemm1_fuse(L, p1x);
    const std::vector<split::Prod> pr1 = make_prods(p1x, fuse1);
    GAIN_TRY(e->prods1.upload(pr1));
    GAIN_TRY(e->H.alloc((size_t)Bpad * L.fpad));
    GAIN_TRY(e->rowerr.alloc(Bpad));
    GAIN_TRY(e->rowerr.zero(st, Bpad));
    if (npieces > 1) {
        GAIN_TRY(e->acc.alloc((size_t)Bpad * L.fpad));
        GAIN_TRY(e->acc.zero(st, (size_t)Bpad * L.fpad));
    }
    const Basis& bFs = e->bases[j->jindF];
    std::vector<split::Tile> t1;
    // first-GEMM refinement counts of the pieces before the last (the counter restarts per piece)
    unsigned long long inexact_prev = 0;
    bool overflow_prev = false;
    for (int piece = 0; piece < npieces; ++piece) {
        if (piece > 0) {   // the next piece's band (the previous GEMM and refinement read theirs)
            GAIN_CUDA(cudaStreamSynchronize(st));
            unsigned int c0 = 0;
            GAIN_CUDA(cudaMemcpy(&c0, e->counters.p, sizeof c0, cudaMemcpyDeviceToHost));
            inexact_prev += c0;
            overflow_prev = overflow_prev || c0 > (unsigned)max_flags;
            GAIN_TRY(load_piece(e, piece));
            GAIN_TRY(launch_layout_band(e, j));
            L.dip_version = e->dip_version;
            L.beta1 = 0;
            GAIN_TRY(band_digits());
            GAIN_CUDA(cudaMemsetAsync(e->counters.p, 0, sizeof(unsigned int), st));
        }
        if (npieces > 1) GAIN_CUDA(cudaMemsetAsync(e->H.p, 0, sizeof(double) * (size_t)Bpad * L.fpad, st));
        t1.clear();
        for (auto& fb : L.fblocks)
            for (int n0 = fb.first; n0 < fb.second; n0 += split::BN) {
                if (npieces > 1) {   // only column tiles holding an upper function of this piece
                    bool any = false;
                    for (int r = n0; r < n0 + split::BN && r < L.fpad && !any; ++r) {
                        if (L.symband) {
                            for (int q = L.fr_ptr[r]; q < L.fr_ptr[r + 1] && !any; ++q)
                                any = bFs.vib[L.fr_col[q]] >= e->startF && bFs.vib[L.fr_col[q]] < e->endF;
                        } else {
                            const int fp = L.f_prim[r];
                            any = fp >= 0 && bFs.vib[fp] >= e->startF && bFs.vib[fp] < e->endF;
                        }
                    }
                    if (!any) continue;
                }
                for (int m0 = 0; m0 < Bpad; m0 += mstep) {
                    split::Tile t;
                    memset(&t, 0, sizeof t);
                    t.m0 = m0;
                    t.n0 = n0;
                    t.a_k0 = L.band_k0[n0];
                    t.b_k0 = 0;
                    t.nkb = L.band_len[n0] / split::BK;
                    t1.push_back(t);
                }
            }
        row_grouped(t1, mstep);
        {   // band tiles of the edge K blocks are shorter: dealt in list order to the unit that
            // frees up first, no unit runs a tile more than the rest (a static round robin of
            // the list left the last units up to two thirds of a tile behind)
            const double per_kb = (double)pr1.size() / p1x.chunks;
            std::vector<double> c1(t1.size());
            for (size_t i = 0; i < t1.size(); ++i) c1[i] = t1[i].nkb * per_kb + 2.0 * (double)pr1.size();
            t1 = list_schedule(t1, c1, pair ? e->num_sms / 2 : e->num_sms);
        }
        GAIN_TRY(e->tiles1.upload(t1));
        split::GemmArgs g1;
        memset(&g1, 0, sizeof g1);
        g1.tiles = e->tiles1.p;
        g1.ntiles = (int)t1.size();
        g1.prods = e->prods1.p;
        g1.nprods = (int)pr1.size();
        g1.nchunks = p1x.chunks;
        g1.beta = p1x.beta;
        g1.slices = p1x.slices;
        g1.out = e->H.p;
        g1.ldo = L.fpad;
        g1.A = e->Vst.view(false);
        g1.B = L.bandStats.view(false);
        g1.c_fix = fix_const((int)pr1.size());
        g1.c_f64 = (float)((double)(L.W + 64) * std::ldexp(1.0, -53) * 1.01);
        g1.rowerr2 = e->rowerr.p;
        g1.flag_mode = 2;   // every H entry FP64-grade, else recomputed in FP64
        g1.tol = (float)tol;
        g1.flags = e->flags1.p;
        g1.nflags = e->counters.p + 0;
        g1.max_flags = max_flags;
        g1.rows_valid = B;
        g1.cols_valid = L.fpad;
        g1.err = e->err.p;
        g1.fuse = fuse1;
        if (piece == 0) GAIN_CUDA(cudaEventRecord(e->ev[2], st));
        if (!t1.empty()) {
            GAIN_CUDA(split::launch_gemm(tmV, pair ? L.tmBandPair : L.tmBand, g1, e->num_sms, st, pair));
            ++e->launches;
        }
        if (piece == npieces - 1) GAIN_CUDA(cudaEventRecord(e->ev[3], st));
        if (piece == 0) {
            // ---- upper vectors -> digits on the low-priority second stream (rows [r0, r1))
            auto slice_upper = [&](int r0, int r1) -> gain_status {
                if (L.general)   // symmetric functions in their own order
                    return slice(e, EF.d.p, EF.nsize, e->d_upper.p + r0, r1 - r0, L.nsymF, nullptr, nullptr, K2, Nupad,
                                 e->Udig.p, p2, e->Ust, false, nullptr, nullptr, e->st2, nullptr, 0, r0);
                return slice(e, EF.d.p, EF.nsize, e->d_upper.p + r0, r1 - r0, EF.nsize, L.d_colposF.p, &L.colposF,
                             L.fpad, Nupad, e->Udig.p, p2, e->Ust, false, nullptr, nullptr, e->st2, L.d_f_sym.p, 0, r0);
            };
            GAIN_CUDA(cudaStreamWaitEvent(e->st2, e->ev[6], 0));
            if (Nu2 > 0) {
                GAIN_CUDA(cudaStreamWaitEvent(e->st2, EF.ready_head, 0));
                GAIN_TRY(slice_upper(0, Nu2));
                GAIN_CUDA(cudaEventRecord(e->ev[9], e->st2));
            }
            if (EF.ready) GAIN_CUDA(cudaStreamWaitEvent(e->st2, EF.ready, 0));
            GAIN_TRY(slice_upper(Nu2, Nu));
            GAIN_CUDA(cudaEventRecord(e->ev[7], e->st2));
        }
        // inexact first-GEMM entries recomputed in FP64
        split::RefineHArgs rh;
        rh.flags = e->flags1.p;
        rh.nflags = e->counters.p + 0;
        rh.max_flags = max_flags;
        rh.vecs = L.general ? e->primI.p : EI.d.p;
        rh.nsize = L.general ? bIs.dimen : EI.nsize;
        rh.row_level = L.general ? e->iota.p : e->d_lower.p;
        rh.i_sym = L.d_i_sym.p;
        rh.band_k0 = L.d_band_k0.p;
        rh.band_len = L.d_band_len.p;
        rh.band = L.band.p;
        rh.W = L.W;
        rh.H = e->H.p;
        rh.ldh = L.fpad;
        rh.eA = e->Vst.e.p;
        rh.rowerr2 = e->rowerr.p;
        GAIN_CUDA(split::launch_refine_h(rh, 2 * e->num_sms, st));
        ++e->launches;
        if (npieces > 1) {
            GAIN_CUDA(launch_add(e->acc.p, e->H.p, (long)Bpad * L.fpad, st));
            ++e->launches;
        }
    }
    if (npieces > 1)
        GAIN_CUDA(cudaMemcpyAsync(e->H.p, e->acc.p, sizeof(double) * (size_t)Bpad * L.fpad, cudaMemcpyDeviceToDevice, st));
    // ---- mixing expansion: H_sym = H_prim T_F (FP64), row error bounds carried over
    const double* Hs = e->H.p;
    if (L.general) {
        GAIN_TRY(e->Hsym.alloc((size_t)Bpad * K2));
        GAIN_CUDA(launch_contract_rowerr(B, e->H.p, L.fpad, L.fpad, e->rowerr.p, e->Vst.e.p, L.sigmaF, L.gamF, st));
        ++e->launches;
        GAIN_CUDA(launch_contract(L.nsymF, L.d_cF_ptr.p, L.d_cF_col.p, L.d_cF_val.p, e->H.p, L.fpad, e->Hsym.p, K2, B,
                                  st));
        ++e->launches;
        Hs = e->Hsym.p;
    }

    // ---- H -> digits; the upper digits (second stream) must be ready before the second GEMM
    GAIN_TRY(slice(e, Hs, K2, nullptr, B, L.general ? L.nsymF : L.fpad, nullptr, nullptr, K2, Bpad, e->Hdig.p, p2,
                   e->Hst, true, e->rowerr.p, e->Vst.e.p, st));
    // the upper digits the (first) amplitude GEMM reads
    GAIN_CUDA(cudaStreamWaitEvent(st, Nu2 > 0 ? e->ev[9] : e->ev[7], 0));
    if (!split::make_digit_map(&tmH, e->Hdig.p, K2, Bpad, p2.slices) ||
        !split::make_digit_map(&tmU, e->Udig.p, K2, Nupad, p2.slices, pair ? split::BN / 2 : split::BM))
        return set_error(GAIN_ERR_CUDA, "cuTensorMapEncodeTiled failed (second GEMM digits)");

    // ---- GEMM 2: amp = H U^T
    std::vector<split::Tile> t2;
    for (int n0 = 0; n0 < Nupad; n0 += split::BN)
        for (int m0 = 0; m0 < Bpad; m0 += mstep) {
            split::Tile t;
            memset(&t, 0, sizeof t);
            t.m0 = m0;
            t.n0 = n0;
            t.a_k0 = 0;
            t.b_k0 = 0;
            t.nkb = K2 / split::BK;
            t2.push_back(t);
        }
    row_grouped(t2, mstep, [&](const split::Tile& t) { return Nu2 > 0 && t.n0 >= Nu2 ? 1 : 0; });
    const std::vector<split::Prod> pr2 = make_prods(p2);
    GAIN_TRY(e->tiles2.upload(t2));
    GAIN_TRY(e->prods2.upload(pr2));
    GAIN_TRY(e->amp.alloc((size_t)Bpad * Nupad));
    GAIN_TRY(e->ampbnd.alloc((size_t)Bpad * Nupad));
    split::GemmArgs g2;
    memset(&g2, 0, sizeof g2);
    g2.tiles = e->tiles2.p;
    g2.ntiles = (int)t2.size();
    g2.prods = e->prods2.p;
    g2.nprods = (int)pr2.size();
    g2.nchunks = p2.chunks;
    g2.beta = p2.beta;
    g2.slices = p2.slices;
    g2.out = e->amp.p;
    g2.ldo = Nupad;
    g2.A = e->Hst.view(false);   // H is FP64-grade: its error is the FP64 method's own
    g2.B = e->Ust.view(false);
    g2.c_fix = fix_const((int)pr2.size());
    g2.c_f64 = (float)((double)((L.general ? L.nsymF : L.nF) + 64) * std::ldexp(1.0, -53) * 1.01);
    g2.rowerr2 = nullptr;
    g2.absmax = e->ull.p + 2;
    g2.flag_mode = 1;
    g2.tol = (float)tol;
    g2.flags = e->flags2.p;
    g2.nflags = e->counters.p + 1;
    g2.max_flags = max_flags;
    g2.rows_valid = B;
    g2.cols_valid = Nu;
    g2.err = e->err.p;
    g2.bnd = e->ampbnd.p;
    g2.ldb = Nupad;
    GAIN_CUDA(cudaEventRecord(e->ev[4], st));
    if (Nu2 > 0) {
        // tiles are upper-block-major: those of the first half (n0 < Nu2) come first
        int n1 = 0;
        while (n1 < (int)t2.size() && t2[n1].n0 < Nu2) ++n1;
        split::GemmArgs ga = g2, gb = g2;
        ga.ntiles = n1;
        gb.tiles = e->tiles2.p + n1;
        gb.ntiles = (int)t2.size() - n1;
        GAIN_CUDA(split::launch_gemm(tmH, tmU, ga, e->num_sms, st, pair));
        GAIN_CUDA(cudaStreamWaitEvent(st, e->ev[7], 0));
        GAIN_CUDA(split::launch_gemm(tmH, tmU, gb, e->num_sms, st, pair));
        e->launches += 2;
    } else {
        GAIN_CUDA(split::launch_gemm(tmH, tmU, g2, e->num_sms, st, pair));
        ++e->launches;
    }
    GAIN_CUDA(cudaEventRecord(e->ev[5], st));
    split::RefineAmpArgs ra;
    ra.flags = e->flags2.p;
    ra.nflags = e->counters.p + 1;
    ra.max_flags = max_flags;
    ra.U = EF.d.p;
    ra.nsize = EF.nsize;
    ra.col_level = e->d_upper.p;
    ra.colpos = L.general ? L.d_ident.p : L.d_colposF.p;
    ra.H = Hs;
    ra.ldh = K2;
    ra.h_inerr = e->Hst.inerr.p;
    ra.eH = e->Hst.e.p;
    ra.amp = e->amp.p;
    ra.lda = Nupad;
    ra.bnd = e->ampbnd.p;
    ra.ldb = Nupad;
    ra.tol = tol;
    ra.absmax = e->ull.p + 2;
    ra.amp_floor = std::sqrt((opts && opts->s_floor > 0) ? opts->s_floor : 1e-10);
    ra.uncertified = e->ull.p;
    ra.uncertified_weak = e->ull.p + 3;
    GAIN_CUDA(split::launch_refine_amp(ra, 4 * e->num_sms, st));
    ++e->launches;
    GAIN_CUDA(cudaEventRecord(e->ev[1], st));

    unsigned int cnt[4];
    unsigned long long unc[4];
    int errw = 0;
    {   // the run's counters through one page-locked area
        if (!e->readback) GAIN_CUDA(cudaMallocHost(&e->readback, 128));
        char* rb = (char*)e->readback;
        GAIN_CUDA(cudaMemcpyAsync(rb, e->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, st));
        GAIN_CUDA(cudaMemcpyAsync(rb + 32, e->ull.p, sizeof unc, cudaMemcpyDeviceToHost, st));
        GAIN_CUDA(cudaMemcpyAsync(rb + 64, e->err.p, sizeof errw, cudaMemcpyDeviceToHost, st));
        GAIN_CUDA(cudaStreamSynchronize(st));
        memcpy(cnt, rb, sizeof cnt);
        memcpy(unc, rb + 32, sizeof unc);
        memcpy(&errw, rb + 64, sizeof errw);
    }
    e->amp_rows = B;
    e->amp_cols = Nu;
    e->amp_ld = Nupad;
    // a refinement list that overflowed in any piece leaves entries unrefined: such a run's
    // amplitudes are not served
    const bool overflow = overflow_prev || cnt[0] > (unsigned)max_flags || cnt[1] > (unsigned)max_flags;
    e->have_amp = errw == 0 && !overflow;
    e->have_bnd = e->have_amp;
    if (stats) {
        memset(stats, 0, sizeof *stats);
        float ms = 0.f, g1ms = 0.f, g2ms = 0.f;
        cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]);
        cudaEventElapsedTime(&g1ms, e->ev[2], e->ev[3]);
        cudaEventElapsedTime(&g2ms, e->ev[4], e->ev[5]);
        stats->device_ms = ms;
        stats->gemm1_ms = g1ms;
        stats->gemm2_ms = g2ms;
        stats->rows = B;
        stats->cols = Nu;
        stats->refined = (long long)std::min<unsigned>(cnt[1], (unsigned)max_flags) +
                         (long long)std::min<unsigned>(cnt[0], (unsigned)max_flags) +
                         (long long)std::min<unsigned long long>(inexact_prev, (unsigned long long)max_flags * (npieces - 1));
        stats->uncertified = (long long)unc[0];
        stats->uncertified_weak = (long long)unc[3];
        stats->amp_max = __builtin_bit_cast(double, unc[2]);
        stats->inexact = (long long)cnt[0] + (long long)inexact_prev;
        stats->beta1 = p1x.beta;
        stats->slices1 = p1x.slices;
        stats->chunks1 = p1x.chunks;
        stats->beta2 = p2.beta;
        stats->slices2 = p2.slices;
        stats->chunks2 = p2.chunks;
        stats->products1 = (int)pr1.size();
        stats->products2 = (int)pr2.size();
        stats->kernel_launches = e->launches - launches0;
        double f = 0;
        // a tile covers mstep rows (256 for CTA pairs); t1 holds the last piece's tiles
        for (auto& t : t1) f += 2.0 * mstep * split::BN * split::BK * (double)t.nkb * pr1.size() / p1x.chunks;
        for (auto& t : t2) f += 2.0 * mstep * split::BN * split::BK * (double)t.nkb * pr2.size() / p2.chunks;
        stats->tensor_flops = f;
    }
    if (errw != 0)
        return set_error(GAIN_ERR_TIMEOUT, "a bounded device wait of the tensor-core GEMM gave up (code %d)", errw);
    if (overflow)
        return set_error(GAIN_ERR_TOL_NOT_MET, "more lines need FP64 refinement than the refinement list holds");
    return GAIN_OK;
}

// The identity of a block-pair job (its blocks and level lists).
// A job and the degenerate components its amplitudes belong to.
std::vector<int> job_key(const gain_pair_job* j, int dI = 0, int dF = 0) {
    std::vector<int> k = {j->jindI, j->gammaI, j->jindF, j->gammaF, j->nlower, j->nupper, dI, dF};
    k.insert(k.end(), j->lower_levels, j->lower_levels + j->nlower);
    k.insert(k.end(), j->upper_levels, j->upper_levels + j->nupper);
    return k;
}

// Inputs changed: the stored amplitudes (adjoint reuse, component slots) no longer apply.
void clear_amp_jobs(gain_engine e) {
    e->amp_job.clear();
    e->deg_job.clear();
    e->deg_filled = 0;
}

// Output.cpp constants (ACOEF, CMCOEF, the radiation constant of beta) and the INTENSITY
// block's parameters for one (J'', J') pair.
LineParams line_params(const gain_line_params* prm, int jI, int jF, bool with_intensity) {
    LineParams p;
    p.acoef_2jI1 = 3.13618923e-7 * (double)(2 * jI + 1);
    p.cmcoef = 1.327209365e-12;
    p.gnsF = prm->gnsF;
    p.two_jF1 = 2.0 * (double)jF + 1.0;
    p.beta = 6.62606896e-27 * 2.99792458e+10 / (1.380658e-16 * prm->temperature);
    p.zpe = prm->zpe;
    p.q_part = prm->q_part;
    p.thresh = prm->thresh;
    p.freq_lo = prm->freq_lo;
    p.freq_hi = prm->freq_hi;
    p.with_intensity = with_intensity;
    p.nslot = 0;
    p.ndegI = 1;
    p.reduced_deg = 0;
    p.slot_stride = 0;
    for (int i = 0; i < kMaxDegSlots; ++i) p.slot[i] = 0;
    return p;
}

// The amplitudes the line assembly reads for prm's degeneracies: the last run (ndegI = ndegF
// = 1), or the component slots gain_run_pair_component filled for the last run's job, in
// Output.cpp's order (idegF outer, idegI inner).
gain_status line_source(gain_engine e, const gain_line_params* prm, LineParams& p, const double** amp, long* ld) {
    if (prm->ndegI < 1 || prm->ndegF < 1 || prm->ndegI > e->maxdeg || prm->ndegF > e->maxdeg)
        return set_error(GAIN_ERR_INVALID_ARG, "degeneracies (%d, %d) outside 1..%d", prm->ndegI, prm->ndegF,
                         e->maxdeg);
    if (prm->ndegI == 1 && prm->ndegF == 1) {
        *amp = e->amp.p;
        *ld = e->amp_ld;
        return GAIN_OK;
    }
    const bool same = e->amp_job.size() >= 8 && e->deg_job.size() == e->amp_job.size() &&
                      std::equal(e->amp_job.begin(), e->amp_job.begin() + 6, e->deg_job.begin()) &&
                      std::equal(e->amp_job.begin() + 8, e->amp_job.end(), e->deg_job.begin() + 8);
    if (!same || !e->deg_filled)
        return set_error(GAIN_ERR_NOT_READY, "degenerate lines: run the component pairs of this job first "
                                             "(gain_run_pair_component / gain_run_pair_degenerate)");
    const int md = e->maxdeg;
    for (int dF = 0; dF < prm->ndegF; ++dF)
        for (int dI = 0; dI < prm->ndegI; ++dI) {
            const int slot = dI + dF * md;
            if (e->deg_filled & (1u << slot)) p.slot[p.nslot++] = slot;
        }
    if (!p.nslot) return set_error(GAIN_ERR_NOT_READY, "no component slot inside the degeneracies");
    p.ndegI = prm->ndegI;
    p.reduced_deg = prm->reduced && prm->ndegI != 1 && prm->ndegF != 1;
    p.slot_stride = (long)e->amp_rows * e->amp_cols;
    *amp = e->deg_amp.p;
    *ld = e->amp_cols;
    return GAIN_OK;
}

}  // namespace
}  // namespace gain

// Every resource of an engine, whatever of it exists (also a partly created one).
void destroy_engine(gain_engine e) {
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->lines_pending) cudaEventSynchronize(e->ev_lines_d2h);
    cudaStreamSynchronize(e->st);
    if (e->st2) cudaStreamSynchronize(e->st2);
    if (e->stc) cudaStreamSynchronize(e->stc);
    if (e->std2h) cudaStreamSynchronize(e->std2h);
    for (auto& ev : e->ev)
        if (ev) cudaEventDestroy(ev);
    if (e->ev_up) cudaEventDestroy(e->ev_up);
    if (e->ev_lines) cudaEventDestroy(e->ev_lines);
    if (e->ev_lines_d2h) cudaEventDestroy(e->ev_lines_d2h);
    if (e->std2h) cudaStreamDestroy(e->std2h);
    if (e->stc) cudaStreamDestroy(e->stc);
    if (e->st2) cudaStreamDestroy(e->st2);
    if (e->st) cudaStreamDestroy(e->st);
    if (e->readback) cudaFreeHost(e->readback);
    delete e;
}

// ====================================================================== C ABI
using namespace gain;

extern "C" {

const char* gain_last_error_string(void) { return gain::g_last_error.c_str(); }

const char* gain_status_string(gain_status s) {
    switch (s) {
        case GAIN_OK: return "GAIN_OK";
        case GAIN_ERR_INVALID_ARG: return "GAIN_ERR_INVALID_ARG";
        case GAIN_ERR_OOM: return "GAIN_ERR_OOM";
        case GAIN_ERR_CUDA: return "GAIN_ERR_CUDA";
        case GAIN_ERR_TIMEOUT: return "GAIN_ERR_TIMEOUT";
        case GAIN_ERR_TOL_NOT_MET: return "GAIN_ERR_TOL_NOT_MET";
        case GAIN_ERR_NOT_READY: return "GAIN_ERR_NOT_READY";
        case GAIN_ERR_UNSUPPORTED: return "GAIN_ERR_UNSUPPORTED";
    }
    return "GAIN_ERR_UNKNOWN";
}

int gain_abi_version(void) { return GAIN_ABI_VERSION; }

gain_status gain_hls_kblock(int dimenF, int dimenI, int jI, int jF, int kF, const int* tauI, const int* tauF,
                            const int* icorrI, const int* icorrF, int startF_idx, int startI_idx,
                            int startFblock, int endFblock, int ncontrF, int kFBlocksize,
                            const int* kblock_size, const double* dipole_me, const double* vector,
                            const double* threej, double* half_ls, int jmax, int dip_stride, void* stream) {
    clear_error();
    (void)kFBlocksize;
    if (dimenF < 0 || dimenI < 0 || jI < 0 || jF < 0 || kF < 0 || kF > jF || jI > jmax || jF > jmax ||
        std::abs(jI - jF) > 1 || ncontrF <= 0 || dip_stride <= 0 || startF_idx < 0 || startI_idx < 0)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_hls_kblock: inconsistent sizes");
    if (dimenF > 0 && (!tauI || !tauF || !icorrI || !icorrF || !kblock_size || !dipole_me || !vector ||
                       !threej || !half_ls))
        return set_error(GAIN_ERR_INVALID_ARG, "gain_hls_kblock: NULL pointer");
    GAIN_CUDA(launch_hls_kblock(dimenF, dimenI, jI, jF, kF, tauI, tauF, icorrI, icorrF, startF_idx,
                                startI_idx, startFblock, endFblock, ncontrF, kblock_size, dipole_me,
                                vector, threej, half_ls, jmax, dip_stride, (cudaStream_t)stream));
    return GAIN_OK;
}

gain_status gain_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int sym_max_degen, const int* kI,
                            const int* kF, const int* ktauI, const int* ktauF, const int* icorrI, const int* icorrF,
                            int startFblock, int endFblock, int ncontrF, const double* dipole_me, const double* wigner,
                            const double* vector, double* half_ls, int dip_stride, void* stream) {
    clear_error();
    if (dimenF < 0 || dimenI < 0 || nlevelI <= 0 || nlevelF <= 0 || sym_max_degen <= 0 || ncontrF <= 0 ||
        dip_stride <= 0 || startFblock < 0 || endFblock < startFblock)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_hls_rotsym: inconsistent sizes");
    if (dimenF > 0 && (!kI || !kF || !ktauI || !ktauF || !icorrI || !icorrF || !dipole_me || !wigner ||
                       !vector || !half_ls))
        return set_error(GAIN_ERR_INVALID_ARG, "gain_hls_rotsym: NULL pointer");
    GAIN_CUDA(launch_hls_rotsym(dimenF, dimenI, nlevelI, nlevelF, sym_max_degen, kI, kF, ktauI, ktauF, icorrI,
                                icorrF, startFblock, endFblock, ncontrF, dipole_me, dip_stride, wigner, vector,
                                half_ls, (cudaStream_t)stream));
    return GAIN_OK;
}

gain_status gain_expand(int dimenI, int igammaI, int maxcoeff, int idegI, int sdeg, int Ntot,
                        const int* ijterms, const int* icontr, const int* N, const double* repres,
                        const double* vecI, double* vec, void* stream) {
    clear_error();
    if (dimenI < 0 || igammaI < 0 || maxcoeff <= 0 || idegI < 0 || sdeg <= 0 || Ntot < 0 || idegI >= sdeg)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_expand: inconsistent sizes");
    if (dimenI > 0 && (!ijterms || !icontr || !N || !repres || !vecI || !vec))
        return set_error(GAIN_ERR_INVALID_ARG, "gain_expand: NULL pointer");
    GAIN_CUDA(launch_expand(dimenI, igammaI, maxcoeff, idegI, sdeg, Ntot, ijterms, icontr, N, repres, vecI,
                            vec, (cudaStream_t)stream));
    return GAIN_OK;
}

gain_status gain_dot(int n, const double* x, const double* y, double* result, void* stream) {
    clear_error();
    if (n < 0 || !result || (n > 0 && (!x || !y))) return set_error(GAIN_ERR_INVALID_ARG, "gain_dot: bad argument");
    GAIN_CUDA(launch_dot(n, x, y, result, (cudaStream_t)stream));
    return GAIN_OK;
}

gain_status gain_threej_table(int jmax, double* table) {
    clear_error();
    if (jmax < 0 || jmax > 200 || !table) return set_error(GAIN_ERR_INVALID_ARG, "gain_threej_table: bad argument");
    threej_table_host(jmax, table);
    return GAIN_OK;
}

gain_status gain_engine_create(int device, int jmax, int nsym, int maxdeg, gain_engine* out) {
    clear_error();
    if (!out || jmax < 0 || jmax > 200 || nsym <= 0 || maxdeg <= 0 || maxdeg * maxdeg > kMaxDegSlots)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_engine_create: bad argument (maxdeg 1..3)");
    *out = nullptr;
    int ndev = 0;
    GAIN_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return set_error(GAIN_ERR_INVALID_ARG, "no CUDA device %d", device);
    GAIN_CUDA(cudaSetDevice(device));
    // a failure below releases what was created so far (streams, events, memory)
    std::unique_ptr<gain_engine_s, void (*)(gain_engine)> e(new gain_engine_s(), destroy_engine);
    e->device = device;
    e->jmax = jmax;
    e->nsym = nsym;
    e->maxdeg = maxdeg;
    GAIN_CUDA(cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, device));
    GAIN_CUDA(cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking));
    {
        int lo = 0, hi = 0;   // numerically larger = lower priority
        GAIN_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        GAIN_CUDA(cudaStreamCreateWithPriority(&e->st2, cudaStreamNonBlocking, lo));
    }
    GAIN_CUDA(cudaStreamCreateWithFlags(&e->stc, cudaStreamNonBlocking));
    GAIN_CUDA(cudaStreamCreateWithFlags(&e->std2h, cudaStreamNonBlocking));
    GAIN_CUDA(cudaEventCreateWithFlags(&e->ev_lines, cudaEventDisableTiming));
    GAIN_CUDA(cudaEventCreateWithFlags(&e->ev_lines_d2h, cudaEventDisableTiming));
    for (auto& ev : e->ev) GAIN_CUDA(cudaEventCreate(&ev));
    GAIN_CUDA(cudaEventCreateWithFlags(&e->ev_up, cudaEventDisableTiming));
    std::vector<double> t((size_t)(jmax + 1) * (jmax + 1) * 9);
    threej_table_host(jmax, t.data());
    GAIN_TRY(e->d3j.upload(t));
    *out = e.release();
    return GAIN_OK;
}

gain_status gain_engine_destroy(gain_engine e) {
    clear_error();
    destroy_engine(e);
    return GAIN_OK;
}

gain_status gain_upload_basis(gain_engine e, int jind, int J, int dimen, const int* K, const int* tau,
                              const int* vib, const int* kblock_size, const int* kstart) {
    clear_error();
    GAIN_TRY(check_engine(e));
    clear_amp_jobs(e);   // inputs changed: no reuse of earlier amplitudes
    if (jind < 0 || jind > 1000 || J < 0 || J > e->jmax || dimen <= 0 || !K || !tau || !vib || !kblock_size || !kstart)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_basis: bad argument");
    // K-sorted, K-blocks consistent with the per-function K (TroveBasisSet.cpp:659-681)
    int pos = 0;
    for (int k = 0; k <= J; ++k) {
        if (kstart[k] != pos || kblock_size[k] < 0) return set_error(GAIN_ERR_INVALID_ARG, "inconsistent kstart at K=%d", k);
        for (int i = 0; i < kblock_size[k]; ++i)
            if (pos + i >= dimen || K[pos + i] != k)
                return set_error(GAIN_ERR_INVALID_ARG, "function %d is not in K block %d", pos + i, k);
        pos += kblock_size[k];
    }
    if (pos != dimen) return set_error(GAIN_ERR_INVALID_ARG, "K blocks cover %d of %d functions", pos, dimen);
    for (int i = 0; i < dimen; ++i)
        if (vib[i] < 0 || tau[i] < 0) return set_error(GAIN_ERR_INVALID_ARG, "negative tau or vibrational index");
    if ((int)e->bases.size() <= jind) {
        e->bases.resize(jind + 1);
        e->infl.resize(jind + 1);
    }
    Basis& b = e->bases[jind];
    b.J = J;
    b.dimen = dimen;
    b.K.assign(K, K + dimen);
    b.tau.assign(tau, tau + dimen);
    b.lev = b.tau;
    for (auto& t : b.tau) t &= 1;
    b.vib.assign(vib, vib + dimen);
    b.kblock.assign(kblock_size, kblock_size + J + 1);
    b.kstart.assign(kstart, kstart + J + 1);
    GAIN_TRY(b.dK.upload(b.K));
    GAIN_TRY(b.dtau.upload(b.tau));
    GAIN_TRY(b.dlev.upload(b.lev));
    GAIN_TRY(b.dvib.upload(b.vib));
    GAIN_TRY(b.dkblock.upload(b.kblock));
    b.present = true;
    e->layouts.clear();
    ++e->struct_version;
    e->cur = nullptr;
    e->plain.key[0] = -1;
    if (e->infl[jind].present)
        for (auto& m : e->infl[jind].maps) m->built = false;
    return GAIN_OK;
}

gain_status gain_upload_inflation(gain_engine e, int jind, const int* icontr, const int* ijterms, int dimen,
                                  int maxcoeff, int matsize, const int* const* N, const double* const* repres,
                                  const int* Ntot, const int* sdeg) {
    clear_error();
    GAIN_TRY(check_engine(e));
    clear_amp_jobs(e);   // inputs changed: no reuse of earlier amplitudes
    if (jind < 0 || jind >= (int)e->bases.size() || !e->bases[jind].present)
        return set_error(GAIN_ERR_NOT_READY, "upload the basis of jind %d first", jind);
    if (dimen != e->bases[jind].dimen || maxcoeff <= 0 || matsize <= 0 || !icontr || !ijterms || !N || !repres ||
        !Ntot || !sdeg)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_inflation: bad argument");
    Inflation& inf = e->infl[jind];
    inf.dimen = dimen;
    inf.maxcoeff = maxcoeff;
    inf.matsize = matsize;
    inf.icontr.assign(icontr, icontr + 2 * (size_t)dimen);
    inf.ijterms.assign(ijterms, ijterms + (size_t)maxcoeff * e->nsym);
    inf.Ntot.assign(Ntot, Ntot + e->nsym);
    inf.sdeg.assign(sdeg, sdeg + e->nsym);
    inf.N.clear();
    inf.repres.clear();
    inf.dN.clear();
    inf.drepres.clear();
    inf.maps.clear();
    for (int r = 0; r < dimen; ++r)
        if (inf.icontr[r] < 0 || inf.icontr[r] >= maxcoeff || inf.icontr[r + dimen] < 0)
            return set_error(GAIN_ERR_INVALID_ARG, "icontr entry %d out of range", r);
    for (int g = 0; g < e->nsym; ++g) {
        if (Ntot[g] < 0 || sdeg[g] <= 0 || !N[g] || (Ntot[g] > 0 && !repres[g]))
            return set_error(GAIN_ERR_INVALID_ARG, "bad expansion table of Gamma %d", g);
        if (sdeg[g] > e->maxdeg)
            return set_error(GAIN_ERR_INVALID_ARG, "Gamma %d: degeneracy %d above the engine's maxdeg %d", g, sdeg[g],
                             e->maxdeg);
        inf.N.emplace_back(N[g], N[g] + maxcoeff);
        const size_t nrep = (size_t)Ntot[g] * sdeg[g] * matsize;
        inf.repres.emplace_back(repres[g], repres[g] + nrep);
        for (int r = 0; r < dimen; ++r) {
            const int irow = inf.icontr[r], ib = inf.icontr[r + dimen];
            const int it = inf.ijterms[irow + g * maxcoeff], n = inf.N[g][irow];
            if (n > 0 && (it < 0 || it + n > Ntot[g] || ib >= matsize))
                return set_error(GAIN_ERR_INVALID_ARG, "expansion of function %d leaves Gamma %d's range", r, g);
        }
        inf.dN.emplace_back(new DevArray<int>());
        inf.drepres.emplace_back(new DevArray<double>());
        GAIN_TRY(inf.dN.back()->upload(inf.N.back()));
        GAIN_TRY(inf.drepres.back()->upload(inf.repres.back()));
        for (int d = 0; d < e->maxdeg; ++d) inf.maps.emplace_back(new GammaMaps());   // [g * maxdeg + ideg]
    }
    GAIN_TRY(inf.dicontr.upload(inf.icontr));
    GAIN_TRY(inf.dijterms.upload(inf.ijterms));
    inf.present = true;
    e->layouts.clear();
    ++e->struct_version;
    e->cur = nullptr;
    e->plain.key[0] = -1;
    return GAIN_OK;
}

gain_status gain_upload_dipole(gain_engine e, const double* piece, int N, int startF, int endF, int ncontrF) {
    clear_error();
    GAIN_TRY(check_engine(e));
    clear_amp_jobs(e);   // inputs changed: no reuse of earlier amplitudes
    if (!piece || N <= 0 || startF < 0 || endF > N || endF - startF != ncontrF || ncontrF <= 0)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_dipole: bad block (N=%d, [%d,%d), ncontrF=%d)", N, startF,
                         endF, ncontrF);
    for (auto& b : e->bases)
        if (b.present)
            for (int v : b.vib)
                if (v >= N) return set_error(GAIN_ERR_INVALID_ARG, "vibrational index %d >= dipole size %d", v, N);
    GAIN_TRY(e->dipole.upload(piece, (size_t)3 * N * ncontrF));
    e->pieces.clear();
    e->piece_loaded = -1;
    e->dipN = N;
    e->startF = startF;
    e->endF = endF;
    e->ncontrF = ncontrF;
    e->dip_present = true;
    ++e->dip_version;
    return GAIN_OK;
}

gain_status gain_upload_dipole_pieces(gain_engine e, int npieces, const double* const* pieces, int N,
                                      const int* startF, const int* endF) {
    clear_error();
    GAIN_TRY(check_engine(e));
    clear_amp_jobs(e);   // inputs changed: no reuse of earlier amplitudes
    if (npieces <= 0 || !pieces || !startF || !endF || N <= 0)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_dipole_pieces: bad argument");
    for (int p = 0; p < npieces; ++p)
        if (!pieces[p] || startF[p] < 0 || endF[p] > N || endF[p] <= startF[p] || (p > 0 && startF[p] < endF[p - 1]))
            return set_error(GAIN_ERR_INVALID_ARG,
                             "gain_upload_dipole_pieces: piece %d [%d,%d) is empty, outside [0,%d) or overlaps", p,
                             startF[p], endF[p], N);
    if (npieces == 1) return gain_upload_dipole(e, pieces[0], N, startF[0], endF[0], endF[0] - startF[0]);
    for (auto& b : e->bases)
        if (b.present)
            for (int v : b.vib)
                if (v >= N) return set_error(GAIN_ERR_INVALID_ARG, "vibrational index %d >= dipole size %d", v, N);
    e->pieces.clear();
    for (int p = 0; p < npieces; ++p) e->pieces.push_back({pieces[p], startF[p], endF[p]});
    e->dipN = N;
    e->dip_present = true;
    e->piece_loaded = -1;
    GAIN_TRY(load_piece(e, 0));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    return GAIN_OK;
}

gain_status gain_upload_wigner(gain_engine e, int jindI, int jindF, int nlevelsI, int nlevelsF, int maxdeg,
                               const double* rot) {
    clear_error();
    GAIN_TRY(check_engine(e));
    clear_amp_jobs(e);   // inputs changed: no reuse of earlier amplitudes
    if (jindI < 0 || jindF < 0 || jindI >= (int)e->bases.size() || jindF >= (int)e->bases.size() || nlevelsI <= 0 ||
        nlevelsF <= 0 || maxdeg <= 0 || !rot)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_wigner: bad argument");
    const Basis& bI = e->bases[jindI];
    const Basis& bF = e->bases[jindF];
    if (!bI.present || !bF.present) return set_error(GAIN_ERR_NOT_READY, "gain_upload_wigner: basis not uploaded");
    if (std::abs(bF.J - bI.J) > 1) return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_wigner: |J' - J''| > 1");
    // in the rotational-symmetry form tau holds the level index and K the degeneracy index
    for (int x = 0; x < bI.dimen; ++x)
        if (bI.lev[x] < 0 || bI.lev[x] >= nlevelsI || bI.K[x] < 0 || bI.K[x] >= maxdeg)
            return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_wigner: lower function %d has level %d / index %d "
                             "outside %d levels x %d", x, bI.lev[x], bI.K[x], nlevelsI, maxdeg);
    for (int x = 0; x < bF.dimen; ++x)
        if (bF.lev[x] < 0 || bF.lev[x] >= nlevelsF || bF.K[x] < 0 || bF.K[x] >= maxdeg)
            return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_wigner: upper function %d has level %d / index %d "
                             "outside %d levels x %d", x, bF.lev[x], bF.K[x], nlevelsF, maxdeg);
    auto& slot = e->wigner[{jindI, jindF}];
    if (!slot) slot.reset(new WignerTab());
    slot->nI = nlevelsI;
    slot->nF = nlevelsF;
    slot->maxdeg = maxdeg;
    GAIN_TRY(slot->rot.upload(rot, (size_t)3 * nlevelsI * nlevelsF * maxdeg * maxdeg));
    slot->version = ++e->wig_version;
    return GAIN_OK;
}

gain_status gain_upload_eigvecs(gain_engine e, int jind, int gamma, int nlevels, int nsize, const double* vecs) {
    clear_error();
    GAIN_TRY(check_engine(e));
    clear_amp_jobs(e);   // inputs changed: no reuse of earlier amplitudes
    if (jind < 0 || gamma < 0 || gamma >= e->nsym || nlevels <= 0 || nsize <= 0 || !vecs)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_eigvecs: bad argument");
    auto& slot = e->eig[{jind, gamma}];
    if (!slot) slot.reset(new Eig());
    if (slot->ready) GAIN_CUDA(cudaEventSynchronize(slot->ready));   // an asynchronous copy into it
    slot->head_rows = 0;
    slot->nlevels = nlevels;
    slot->nsize = nsize;
    GAIN_TRY(slot->d.alloc((size_t)nlevels * nsize));
    // host or device memory (unified addressing tells them apart)
    GAIN_CUDA(cudaMemcpyAsync(slot->d.p, vecs, sizeof(double) * (size_t)nlevels * nsize, cudaMemcpyDefault, e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    return GAIN_OK;
}

gain_status gain_release_eigvecs(gain_engine e, int jind, int gamma) {
    clear_error();
    GAIN_TRY(check_engine(e));
    auto it = e->eig.find({jind, gamma});
    if (it == e->eig.end()) return GAIN_OK;
    GAIN_TRY(gain_lines_wait(e));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st2));
    if (it->second->ready) GAIN_CUDA(cudaEventSynchronize(it->second->ready));
    clear_amp_jobs(e);
    e->eig.erase(it);
    return GAIN_OK;
}

gain_status gain_upload_eigvecs_async(gain_engine e, int jind, int gamma, int nlevels, int nsize,
                                      const double* vecs) {
    clear_error();
    GAIN_TRY(check_engine(e));
    clear_amp_jobs(e);   // inputs changed: no reuse of earlier amplitudes
    if (jind < 0 || gamma < 0 || gamma >= e->nsym || nlevels <= 0 || nsize <= 0 || !vecs)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_upload_eigvecs_async: bad argument");
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, vecs) != cudaSuccess) {
        (void)cudaGetLastError();
        pa.type = cudaMemoryTypeUnregistered;
    }
    // pageable memory cannot be copied asynchronously: the synchronous upload
    if (pa.type != cudaMemoryTypeHost) return gain_upload_eigvecs(e, jind, gamma, nlevels, nsize, vecs);
    auto& slot = e->eig[{jind, gamma}];
    if (!slot) slot.reset(new Eig());
    if (!slot->ready) GAIN_CUDA(cudaEventCreateWithFlags(&slot->ready, cudaEventDisableTiming));
    if (!slot->ready_head) GAIN_CUDA(cudaEventCreateWithFlags(&slot->ready_head, cudaEventDisableTiming));
    GAIN_CUDA(cudaEventSynchronize(slot->ready));   // a previous asynchronous copy into it
    slot->nlevels = nlevels;
    slot->nsize = nsize;
    GAIN_TRY(slot->d.alloc((size_t)nlevels * nsize));
    // after everything already queued on the engine's streams (the second stream's work is
    // joined to the first before each run ends)
    if (!e->ev_up_fresh) GAIN_CUDA(cudaEventRecord(e->ev_up, e->st));   // after all queued work
    GAIN_CUDA(cudaStreamWaitEvent(e->stc, e->ev_up, 0));
    // two parts: a run can start on the upper states of the first part while the second
    // is still arriving
    // (the head ends on a multiple of 128 rows, where the run's upper halves split)
    const int head = nlevels >= 512 ? std::min(nlevels - 1, round_up(nlevels / 2, 128)) : 0;
    if (head > 0) {
        GAIN_CUDA(cudaMemcpyAsync(slot->d.p, vecs, sizeof(double) * (size_t)head * nsize, cudaMemcpyHostToDevice,
                                  e->stc));
        GAIN_CUDA(cudaEventRecord(slot->ready_head, e->stc));
    }
    GAIN_CUDA(cudaMemcpyAsync(slot->d.p + (size_t)head * nsize, vecs + (size_t)head * nsize,
                              sizeof(double) * (size_t)(nlevels - head) * nsize, cudaMemcpyHostToDevice, e->stc));
    GAIN_CUDA(cudaEventRecord(slot->ready, e->stc));
    slot->head_rows = head;
    return GAIN_OK;
}

gain_status gain_adjoint_pair(gain_engine e, const gain_pair_job* job, const double* dL_dS, double* dL_dmu,
                              gain_stats* stats) {
    return gain_adjoint_pair_prec(e, job, dL_dS, dL_dmu, GAIN_ADJOINT_FP64, stats);
}

namespace {
// dL/dmu of one block pair through the adjoint chain, summed over the component pairs comps
// (one pair, (0, 0), for non-degenerate symmetries) with dS/damp = 2 scale amp.  Each pair's
// forward amplitudes: the last run's when it computed this job and pair, a component slot of
// the job, else the plain FP64 path (the reference's method).
// The tensor-core adjoint chain of one component pair after G = dL/damp (FP64 [B][Nu]):
//   dH = G U                 digit GEMM, rows B, columns the upper symmetric functions, inner Nu
//   dh = T_F dH, vp = T_I v  the expansions (FP64)
//   dM = dh^T vp             digit GEMM, rows the upper primitives of the expansion's support
//                            (grouped by K, padded to 128), columns the lower ones (grouped by
//                            K, padded to 64), inner the B lower states; only the band tiles
//   dL/dmu += factor dM      FP64 scatter over the band
// Entries whose exact-accumulation certificate fails are recomputed in FP64.
constexpr int kAdjSplitBits = 48;
gain_status adjoint_split_chain(gain_engine e, const gain_pair_job* job, int dI, int dF, const double* G,
                                double* tflops) {
    using split::BK;
    using split::BM;
    using split::BN;
    const Basis& bI = e->bases[job->jindI];
    const Basis& bF = e->bases[job->jindF];
    Inflation& iI = e->infl[job->jindI];
    Inflation& iF = e->infl[job->jindF];
    const Eig& EI = *e->eig[{job->jindI, job->gammaI}];
    const Eig& EF = *e->eig[{job->jindF, job->gammaF}];
    GammaMaps* mI = gamma_maps(e, job->jindI, job->gammaI, dI);
    GammaMaps* mF = gamma_maps(e, job->jindF, job->gammaF, dF);
    if (!mI || !mF) return GAIN_ERR_OOM;
    const WignerTab* wt = wigner_of(e, job->jindI, job->jindF);
    cudaStream_t st = e->st;
    const int B = job->nlower, Nu = job->nupper, NtF = iF.Ntot[job->gammaF];
    const int Bpad = round_up(B, BM), Bk = round_up(B, BK);
    const int Nuk = round_up(Nu, BK), NtFpad = round_up(NtF, BN);
    const SplitParams pA = choose_params(Nuk, nullptr, kAdjSplitBits, 8);
    const SplitParams pB = choose_params(Bk, nullptr, kAdjSplitBits, 8);
    const int cap = kMaxFlags;
    GAIN_TRY(e->adjs_flags.alloc(cap));
    GAIN_TRY(e->adjs_cnt.alloc(2));
    GAIN_TRY(e->adjs_cnt.zero(st, 2));
    GAIN_TRY(e->adjs_err.alloc(1));
    GAIN_TRY(e->adjs_err.zero(st, 1));
    double fl = 0.0;
    auto zero_dig = [&](int k, size_t n, size_t rows, int nch) -> gain_status {
        GAIN_TRY(e->adjs_dig[k].alloc(n));
        GAIN_TRY(e->adjs_dig[k].zero(st, n));
        GAIN_TRY(e->adjs_st[k].alloc(rows, nch, false));
        GAIN_TRY(e->adjs_st[k].zero(st, rows, nch, false));
        return GAIN_OK;
    };
    // C = A B^T over the listed tiles from digit buffers ka (rowsA rows) and kb (rowsB rows),
    // inner length ldk; the flags of uncertified entries go to the list behind cnt
    auto gemm = [&](int ka, int kb, const SplitParams& p, int ldk, int rowsA, int rowsB, double* out, long ldo,
                    int rows_valid, int cols_valid, const std::vector<split::Tile>& tiles,
                    DevArray<split::Tile>& dtiles, DevArray<split::Prod>& dprods, unsigned int* cnt) -> gain_status {
        CUtensorMap ta, tb;
        if (!split::make_digit_map(&ta, e->adjs_dig[ka].p, ldk, rowsA, p.slices) ||
            !split::make_digit_map(&tb, e->adjs_dig[kb].p, ldk, rowsB, p.slices))
            return set_error(GAIN_ERR_CUDA, "cuTensorMapEncodeTiled failed (adjoint digits)");
        const std::vector<split::Prod> pr = make_prods(p);
        GAIN_TRY(dprods.upload(pr));
        GAIN_TRY(dtiles.upload(tiles));
        split::GemmArgs g;
        memset(&g, 0, sizeof g);
        g.tiles = dtiles.p;
        g.ntiles = (int)tiles.size();
        g.prods = dprods.p;
        g.nprods = (int)pr.size();
        g.nchunks = p.chunks;
        g.beta = p.beta;
        g.slices = p.slices;
        g.out = out;
        g.ldo = ldo;
        g.A = e->adjs_st[ka].view(false);
        g.B = e->adjs_st[kb].view(false);
        g.c_fix = fix_const((int)pr.size());
        g.c_f64 = (float)((double)(ldk + 64) * std::ldexp(1.0, -53) * 1.01);
        g.flag_mode = 0;   // only entries whose exact accumulation is not certified
        g.flags = e->adjs_flags.p;
        g.nflags = cnt;
        g.max_flags = cap;
        g.rows_valid = rows_valid;
        g.cols_valid = cols_valid;
        g.err = e->adjs_err.p;
        GAIN_CUDA(split::launch_gemm(ta, tb, g, e->num_sms, st, false));
        for (auto& t : tiles) fl += 2.0 * BM * BN * BK * t.nkb * (double)pr.size() / p.chunks;
        return GAIN_OK;
    };
    // ---- dH = G U: A = G rows (inner: upper states), B = U^T rows (upper symmetric functions)
    {
        std::vector<int> umap(NtFpad, -1);
        for (int f = 0; f < NtF; ++f) umap[f] = f;
        GAIN_TRY(e->adjs_umap.upload(umap));
        GAIN_TRY(e->adjs_UT.alloc((size_t)NtFpad * Nuk));
        GAIN_CUDA(launch_gather_t(NtFpad, Nu, Nuk, EF.d.p, EF.nsize, e->d_upper.p, e->adjs_umap.p, e->adjs_UT.p, st));
        GAIN_TRY(zero_dig(0, (size_t)pA.slices * Bpad * Nuk, Bpad, pA.chunks));
        GAIN_TRY(zero_dig(1, (size_t)pA.slices * NtFpad * Nuk, NtFpad, pA.chunks));
        GAIN_TRY(slice(e, G, Nu, nullptr, B, Nu, nullptr, nullptr, Nuk, Bpad, e->adjs_dig[0].p, pA, e->adjs_st[0],
                       false, nullptr, nullptr, st));
        GAIN_TRY(slice(e, e->adjs_UT.p, Nuk, nullptr, NtFpad, Nuk, nullptr, nullptr, Nuk, NtFpad, e->adjs_dig[1].p, pA,
                       e->adjs_st[1], false, nullptr, nullptr, st));
        std::vector<split::Tile> t;
        for (int n0 = 0; n0 < NtFpad; n0 += BN)
            for (int m0 = 0; m0 < Bpad; m0 += BM) {
                split::Tile x;
                memset(&x, 0, sizeof x);
                x.m0 = m0;
                x.n0 = n0;
                x.nkb = Nuk / BK;
                t.push_back(x);
            }
        row_grouped(t, BM);
        GAIN_TRY(e->adjs_dH.alloc((size_t)Bpad * NtFpad));
        GAIN_TRY(gemm(0, 1, pA, Nuk, Bpad, NtFpad, e->adjs_dH.p, NtFpad, B, NtF, t, e->adjs_tiles1, e->adjs_prods1,
                      e->adjs_cnt.p));
        GAIN_CUDA(launch_refine_rows(e->adjs_flags.p, e->adjs_cnt.p, cap, G, Nu, e->adjs_UT.p, Nuk, Nu, e->adjs_dH.p,
                                     NtFpad, 2 * e->num_sms, st));
    }
    // ---- dh = T_F dH, vp = T_I v (primitive spaces)
    GAIN_TRY(e->adj_dh.alloc((size_t)B * bF.dimen));
    GAIN_TRY(e->adj_vp.alloc((size_t)B * bI.dimen));
    double* dh = e->adj_dh.p;
    double* vp = e->adj_vp.p;
    GAIN_CUDA(launch_expand_levels(iF.dimen, job->gammaF, iF.maxcoeff, dF, iF.sdeg[job->gammaF], NtF, iF.dijterms.p,
                                   iF.dicontr.p, iF.dN[job->gammaF]->p, iF.drepres[job->gammaF]->p,
                                   (const double*)e->adjs_dH.p, NtFpad, e->adj_iota.p, dh, bF.dimen, B, st));
    GAIN_CUDA(launch_expand_levels(iI.dimen, job->gammaI, iI.maxcoeff, dI, iI.sdeg[job->gammaI], iI.Ntot[job->gammaI],
                                   iI.dijterms.p, iI.dicontr.p, iI.dN[job->gammaI]->p, iI.drepres[job->gammaI]->p,
                                   EI.d.p, EI.nsize, e->d_lower.p, vp, bI.dimen, B, st));
    // ---- the band layout over the expansions' supports, grouped by K
    std::vector<int> fmap, imap, fstart(bF.J + 2, 0), istart(bI.J + 2, 0);
    for (int k = 0; k <= bF.J; ++k) {
        for (int q = mF->sup_start[k]; q < mF->sup_start[k + 1]; ++q) fmap.push_back(mF->support[q]);
        while (fmap.size() % BM) fmap.push_back(-1);
        fstart[k + 1] = (int)fmap.size();
    }
    for (int k = 0; k <= bI.J; ++k) {
        for (int q = mI->sup_start[k]; q < mI->sup_start[k + 1]; ++q) imap.push_back(mI->support[q]);
        while (imap.size() % BK) imap.push_back(-1);
        istart[k + 1] = (int)imap.size();
    }
    const int Fpad = std::max((int)fmap.size(), BM), Ipad = (int)imap.size();
    fmap.resize(Fpad, -1);
    const int ldM = round_up(Ipad + BN, BN);
    imap.resize(ldM, -1);
    std::vector<int> blo(Fpad, 0), bhi(Fpad, 0);
    std::vector<split::Tile> t2;
    for (int k = 0; k <= bF.J; ++k) {
        if (fstart[k + 1] == fstart[k]) continue;
        int lo = 0, hi = Ipad;
        if (!wt) {
            const int klo = std::max(k - 1, 0), khi = std::min(k + 1, bI.J);
            if (klo > khi) continue;
            lo = istart[klo];
            hi = istart[khi + 1];
        }
        if (hi <= lo) continue;
        for (int r = fstart[k]; r < fstart[k + 1]; ++r) {
            blo[r] = lo;
            bhi[r] = hi;
        }
        for (int m0 = fstart[k]; m0 < fstart[k + 1]; m0 += BM)
            for (int n0 = lo; n0 < hi; n0 += BN) {
                split::Tile x;
                memset(&x, 0, sizeof x);
                x.m0 = m0;
                x.n0 = n0;
                x.nkb = Bk / BK;
                t2.push_back(x);
            }
    }
    GAIN_TRY(e->adjs_fmap.upload(fmap));
    GAIN_TRY(e->adjs_imap.upload(imap));
    GAIN_TRY(e->adjs_blo.upload(blo));
    GAIN_TRY(e->adjs_bhi.upload(bhi));
    // ---- dM = dh^T vp on the band: A = dh^T rows (upper positions), B = vp^T rows (lower)
    GAIN_TRY(e->adjs_dhT.alloc((size_t)Fpad * Bk));
    GAIN_TRY(e->adjs_vpT.alloc((size_t)ldM * Bk));
    GAIN_CUDA(launch_gather_t(Fpad, B, Bk, dh, bF.dimen, nullptr, e->adjs_fmap.p, e->adjs_dhT.p, st));
    GAIN_CUDA(launch_gather_t(ldM, B, Bk, vp, bI.dimen, nullptr, e->adjs_imap.p, e->adjs_vpT.p, st));
    GAIN_TRY(zero_dig(2, (size_t)pB.slices * Fpad * Bk, Fpad, pB.chunks));
    GAIN_TRY(zero_dig(3, (size_t)pB.slices * ldM * Bk, ldM, pB.chunks));
    GAIN_TRY(slice(e, e->adjs_dhT.p, Bk, nullptr, Fpad, Bk, nullptr, nullptr, Bk, Fpad, e->adjs_dig[2].p, pB,
                   e->adjs_st[2], false, nullptr, nullptr, st));
    GAIN_TRY(slice(e, e->adjs_vpT.p, Bk, nullptr, ldM, Bk, nullptr, nullptr, Bk, ldM, e->adjs_dig[3].p, pB,
                   e->adjs_st[3], false, nullptr, nullptr, st));
    GAIN_TRY(e->adjs_dM.alloc((size_t)Fpad * ldM));
    if (!t2.empty()) {
        GAIN_TRY(gemm(2, 3, pB, Bk, Fpad, ldM, e->adjs_dM.p, ldM, Fpad, ldM, t2, e->adjs_tiles2, e->adjs_prods2,
                      e->adjs_cnt.p + 1));
        GAIN_CUDA(launch_refine_rows(e->adjs_flags.p, e->adjs_cnt.p + 1, cap, e->adjs_dhT.p, Bk, e->adjs_vpT.p, Bk,
                                     Bk, e->adjs_dM.p, ldM, 2 * e->num_sms, st));
    }
    // ---- dL/dmu from the band
    AdjArgs a;
    memset(&a, 0, sizeof a);
    a.dimF = bF.dimen;
    a.dimI = bI.dimen;
    a.nb = B;
    a.vibF = bF.dvib.p;
    a.vibI = bI.dvib.p;
    a.KF = bF.dK.p;
    a.KI = bI.dK.p;
    a.tauF = bF.dtau.p;
    a.tauI = bI.dtau.p;
    a.levF = bF.dlev.p;
    a.levI = bI.dlev.p;
    a.jI = bI.J;
    a.jF = bF.J;
    a.jmax = e->jmax;
    a.threej = e->d3j.p;
    if (wt) {
        a.wigner = wt->rot.p;
        a.nlevelI = wt->nI;
        a.nlevelF = wt->nF;
        a.maxdeg = wt->maxdeg;
    }
    a.startF = e->startF;
    a.endF = e->endF;
    a.ncontrF = e->ncontrF;
    a.dipN = e->dipN;
    a.dmu = e->adj_dmu.p;
    GAIN_CUDA(launch_adj_scatter_band(a, Fpad, e->adjs_fmap.p, e->adjs_imap.p, e->adjs_blo.p, e->adjs_bhi.p,
                                      e->adjs_dM.p, ldM, st));
    // the refinement lists must have held every flagged entry, and no bounded wait gave up
    unsigned int cnt[2] = {0, 0};
    int errw = 0;
    GAIN_CUDA(cudaMemcpyAsync(cnt, e->adjs_cnt.p, sizeof cnt, cudaMemcpyDeviceToHost, st));
    GAIN_CUDA(cudaMemcpyAsync(&errw, e->adjs_err.p, sizeof errw, cudaMemcpyDeviceToHost, st));
    GAIN_CUDA(cudaStreamSynchronize(st));
    if (errw) return set_error(GAIN_ERR_TIMEOUT, "a bounded device wait of the adjoint GEMM gave up (code %d)", errw);
    if (cnt[0] > (unsigned)cap || cnt[1] > (unsigned)cap)
        return set_error(GAIN_ERR_TOL_NOT_MET, "adjoint: more uncertified products than the refinement list holds");
    if (tflops) *tflops += fl;
    return GAIN_OK;
}

gain_status adjoint_run(gain_engine e, const gain_pair_job* job, const std::vector<std::pair<int, int>>& comps,
                        double scale, const double* dL_dS, double* dL_dmu, gain_adjoint_precision prec,
                        gain_stats* stats) {
    const bool f32 = prec == GAIN_ADJOINT_FP32;
    const bool tc = prec == GAIN_ADJOINT_SPLIT;
    double tflops = 0.0;
    e->ev_up_fresh = false;
    const Basis& bI = e->bases[job->jindI];
    const Basis& bF = e->bases[job->jindF];
    Inflation& iI = e->infl[job->jindI];
    Inflation& iF = e->infl[job->jindF];
    const Eig& EI = *e->eig[{job->jindI, job->gammaI}];
    const Eig& EF = *e->eig[{job->jindF, job->gammaF}];
    const int B = job->nlower, Nu = job->nupper, NtF = iF.Ntot[job->gammaF];
    const size_t nS = (size_t)B * Nu, nmu = (size_t)3 * e->dipN * e->ncontrF;
    cudaStream_t st = e->st;
    GAIN_TRY(e->adj_dLdS.upload(dL_dS, nS));
    // work space in the chain's precision (float arrays live in the double allocations)
    const size_t esz = f32 ? sizeof(float) : sizeof(double);
    auto words = [&](size_t n) { return (n * esz + sizeof(double) - 1) / sizeof(double); };
    GAIN_TRY(e->adj_G.alloc(words(nS)));
    GAIN_TRY(e->adj_dH.alloc(words((size_t)B * NtF)));
    GAIN_TRY(e->adj_dh.alloc(words((size_t)B * bF.dimen)));
    GAIN_TRY(e->adj_vp.alloc(words((size_t)B * bI.dimen)));
    GAIN_TRY(e->adj_dmu.alloc(nmu));
    GAIN_TRY(e->adj_dmu.zero(st, nmu));
    std::vector<int> iota(B);
    for (int b = 0; b < B; ++b) iota[b] = b;
    GAIN_TRY(e->adj_iota.upload(iota));
    // (F, I) tiles that hold a possibly non-zero factor: F in the dipole piece and, in the
    // K-block form, |K_I - K_F| <= 1 somewhere in the tile
    const WignerTab* wt = wigner_of(e, job->jindI, job->jindF);
    const int tl = adj_tile();
    auto kranges = [&](const Basis& b, bool upper, std::vector<int>& lo, std::vector<int>& hi) {
        const int nt = (b.dimen + tl - 1) / tl;
        lo.assign(nt, INT_MAX);
        hi.assign(nt, INT_MIN);
        for (int f = 0; f < b.dimen; ++f) {
            if (upper && (b.vib[f] < e->startF || b.vib[f] >= e->endF)) continue;
            lo[f / tl] = std::min(lo[f / tl], b.K[f]);
            hi[f / tl] = std::max(hi[f / tl], b.K[f]);
        }
    };
    std::vector<int> kFlo, kFhi, kIlo, kIhi, tiles;
    kranges(bF, true, kFlo, kFhi);
    kranges(bI, false, kIlo, kIhi);
    for (size_t tf = 0; tf < kFlo.size(); ++tf) {
        if (kFlo[tf] > kFhi[tf]) continue;   // no function of the piece
        for (size_t ti = 0; ti < kIlo.size(); ++ti) {
            if (!wt && (kIlo[ti] > kFhi[tf] + 1 || kFlo[tf] > kIhi[ti] + 1)) continue;
            tiles.push_back((int)tf * tl);
            tiles.push_back((int)ti * tl);
        }
    }
    GAIN_TRY(e->adj_tiles.upload(tiles));
    void* G = e->adj_G.p;
    void* dH = e->adj_dH.p;
    void* dh = e->adj_dh.p;
    void* vp = e->adj_vp.p;
    const std::vector<int> key = job_key(job);
    double chain_ms = 0.0;
    for (const auto& c : comps) {
        const int dI = c.first, dF = c.second;
        const double* amp = nullptr;
        long ld_amp = 0;
        const int slot = dI + dF * e->maxdeg;
        if (e->have_amp && e->amp_job == job_key(job, dI, dF)) {
            amp = e->amp.p;
            ld_amp = e->amp_ld;
        } else if (e->deg_job == key && (e->deg_filled & (1u << slot))) {
            amp = e->deg_amp.p + (size_t)slot * nS;
            ld_amp = Nu;
        } else {
            // the pair's forward: the split path for the tensor-core adjoint (half line
            // strengths recomputed on the tensor cores), else the FP64 plain path
            e->have_amp = false;
            e->amp_job.clear();
            if (tc) GAIN_TRY(run_split(e, job, dI, dF, nullptr, nullptr));
            else GAIN_TRY(run_plain(e, job, dI, dF, nullptr));
            e->amp_job = job_key(job, dI, dF);
            e->have_amp = true;
            amp = e->amp.p;
            ld_amp = e->amp_ld;
        }
        GAIN_CUDA(cudaEventRecord(e->ev[2], st));
        // dL/damp = dL/dS 2 amp;  dL/dH = G U (upper symmetry space);  dL/dh = T_F dH
        GAIN_CUDA(launch_adj_scale(B, Nu, e->adj_dLdS.p, amp, ld_amp, 2.0 * scale, G, f32, st));
        if (tc) {
            GAIN_TRY(adjoint_split_chain(e, job, dI, dF, (const double*)G, &tflops));
            GAIN_CUDA(cudaEventRecord(e->ev[3], st));
            GAIN_CUDA(cudaEventSynchronize(e->ev[3]));
            float ms = 0.f;
            GAIN_CUDA(cudaEventElapsedTime(&ms, e->ev[2], e->ev[3]));
            chain_ms += ms;
            continue;
        }
        GAIN_CUDA(launch_adj_gemm(B, NtF, Nu, G, Nu, EF.d.p, EF.nsize, e->d_upper.p, dH, NtF, f32, st));
        const int* repF_N = iF.dN[job->gammaF]->p;
        const double* repF = iF.drepres[job->gammaF]->p;
        const int* repI_N = iI.dN[job->gammaI]->p;
        const double* repI = iI.drepres[job->gammaI]->p;
        if (f32) {
            GAIN_CUDA(launch_expand_levels(iF.dimen, job->gammaF, iF.maxcoeff, dF, iF.sdeg[job->gammaF], NtF,
                                           iF.dijterms.p, iF.dicontr.p, repF_N, repF, (const float*)dH, NtF,
                                           e->adj_iota.p, (float*)dh, bF.dimen, B, st));
            GAIN_CUDA(launch_expand_levels(iI.dimen, job->gammaI, iI.maxcoeff, dI, iI.sdeg[job->gammaI],
                                           iI.Ntot[job->gammaI], iI.dijterms.p, iI.dicontr.p, repI_N, repI, EI.d.p,
                                           EI.nsize, e->d_lower.p, (float*)vp, bI.dimen, B, st));
        } else {
            GAIN_CUDA(launch_expand_levels(iF.dimen, job->gammaF, iF.maxcoeff, dF, iF.sdeg[job->gammaF], NtF,
                                           iF.dijterms.p, iF.dicontr.p, repF_N, repF, (const double*)dH, NtF,
                                           e->adj_iota.p, (double*)dh, bF.dimen, B, st));
            // lower vectors in primitive space
            GAIN_CUDA(launch_expand_levels(iI.dimen, job->gammaI, iI.maxcoeff, dI, iI.sdeg[job->gammaI],
                                           iI.Ntot[job->gammaI], iI.dijterms.p, iI.dicontr.p, repI_N, repI, EI.d.p,
                                           EI.nsize, e->d_lower.p, (double*)vp, bI.dimen, B, st));
        }
        // dL/dmu from the band (or dense) products
        AdjArgs a;
        memset(&a, 0, sizeof a);
        a.dimF = bF.dimen;
        a.dimI = bI.dimen;
        a.nb = B;
        a.vibF = bF.dvib.p;
        a.vibI = bI.dvib.p;
        a.KF = bF.dK.p;
        a.KI = bI.dK.p;
        a.tauF = bF.dtau.p;
        a.tauI = bI.dtau.p;
        a.levF = bF.dlev.p;
        a.levI = bI.dlev.p;
        a.jI = bI.J;
        a.jF = bF.J;
        a.jmax = e->jmax;
        a.threej = e->d3j.p;
        if (wt) {
            a.wigner = wt->rot.p;
            a.nlevelI = wt->nI;
            a.nlevelF = wt->nF;
            a.maxdeg = wt->maxdeg;
        }
        a.startF = e->startF;
        a.endF = e->endF;
        a.ncontrF = e->ncontrF;
        a.dipN = e->dipN;
        a.dh = dh;
        a.ld_dh = bF.dimen;
        a.vp = vp;
        a.ld_vp = bI.dimen;
        a.dmu = e->adj_dmu.p;
        GAIN_CUDA(launch_adj_dm(a, e->adj_tiles.p, (int)(tiles.size() / 2), f32, st));
        GAIN_CUDA(cudaEventRecord(e->ev[3], st));
        GAIN_CUDA(cudaEventSynchronize(e->ev[3]));
        float ms = 0.f;
        GAIN_CUDA(cudaEventElapsedTime(&ms, e->ev[2], e->ev[3]));
        chain_ms += ms;
    }
    if (f32) {
        std::vector<float> h(nmu);
        GAIN_CUDA(cudaMemcpyAsync(h.data(), e->adj_dmu.p, sizeof(float) * nmu, cudaMemcpyDeviceToHost, st));
        GAIN_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < nmu; ++i) dL_dmu[i] += (double)h[i];
    } else {
        std::vector<double> h(nmu);
        GAIN_CUDA(cudaMemcpyAsync(h.data(), e->adj_dmu.p, sizeof(double) * nmu, cudaMemcpyDeviceToHost, st));
        GAIN_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < nmu; ++i) dL_dmu[i] += h[i];
    }
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->device_ms = chain_ms;
        stats->rows = B;
        stats->cols = Nu;
        stats->kernel_launches = (tc ? 17 : 5) * (int)comps.size();
        stats->tensor_flops = tflops;
    }
    GAIN_CUDA(cudaEventRecord(e->ev_up, st));
    e->ev_up_fresh = true;
    return GAIN_OK;
}

gain_status adjoint_checks(gain_engine e, const gain_pair_job* job, const double* dL_dS, double* dL_dmu,
                           gain_adjoint_precision prec) {
    if (prec != GAIN_ADJOINT_FP64 && prec != GAIN_ADJOINT_FP32 && prec != GAIN_ADJOINT_SPLIT)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_adjoint_pair_prec: unknown precision %d", (int)prec);
    GAIN_TRY(check_engine(e));
    GAIN_TRY(validate_job(e, job));
    if (!dL_dS || !dL_dmu) return set_error(GAIN_ERR_INVALID_ARG, "gain_adjoint_pair: NULL argument");
    if (e->pieces.size() > 1)
        return set_error(GAIN_ERR_UNSUPPORTED, "gain_adjoint_pair: upload the dipole as one piece");
    return GAIN_OK;
}
}  // namespace

gain_status gain_adjoint_pair_prec(gain_engine e, const gain_pair_job* job, const double* dL_dS, double* dL_dmu,
                                   gain_adjoint_precision prec, gain_stats* stats) {
    clear_error();
    GAIN_TRY(adjoint_checks(e, job, dL_dS, dL_dmu, prec));
    if (e->infl[job->jindI].sdeg[job->gammaI] != 1 || e->infl[job->jindF].sdeg[job->gammaF] != 1)
        return set_error(GAIN_ERR_UNSUPPORTED,
                         "gain_adjoint_pair: degenerate symmetries go through gain_adjoint_pair_degenerate");
    return adjoint_run(e, job, {{0, 0}}, 1.0, dL_dS, dL_dmu, prec, stats);
}

gain_status gain_adjoint_pair_degenerate(gain_engine e, const gain_pair_job* job, const gain_filters* f,
                                         const double* dL_dS, double* dL_dmu, gain_adjoint_precision prec,
                                         gain_stats* stats) {
    clear_error();
    GAIN_TRY(adjoint_checks(e, job, dL_dS, dL_dmu, prec));
    if (!f || !f->sym_degen || f->nsym != e->nsym)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_adjoint_pair_degenerate: filters of %d symmetries needed",
                         e->nsym);
    const int nI = f->sym_degen[job->gammaI], nF = f->sym_degen[job->gammaF];
    if (nI != e->infl[job->jindI].sdeg[job->gammaI] || nF != e->infl[job->jindF].sdeg[job->gammaF])
        return set_error(GAIN_ERR_INVALID_ARG, "sym_degen differs from the expansion tables' degeneracies");
    std::vector<std::pair<int, int>> comps;
    for (int dF = 0; dF < nF; ++dF)
        for (int dI = 0; dI < nI; ++dI)
            if (gain_degeneracy_filter(f, job->gammaI, job->gammaF, dI, dF)) comps.push_back({dI, dF});
    if (comps.empty()) return set_error(GAIN_ERR_INVALID_ARG, "no component pair passes the degeneracy filter");
    // S = sum amp^2 / ndegI, times ndegI when reduced and both states are degenerate
    const double scale = (f->reduced && nI != 1 && nF != 1) ? 1.0 : 1.0 / nI;
    return adjoint_run(e, job, comps, scale, dL_dS, dL_dmu, prec, stats);
}

namespace {
gain_status run_component(gain_engine e, const gain_pair_job* job, int dI, int dF, gain_path path,
                          const gain_split_opts* opts, gain_stats* stats) {
    GAIN_TRY(check_engine(e));
    GAIN_TRY(validate_job(e, job));
    const int sI = e->infl[job->jindI].sdeg[job->gammaI], sF = e->infl[job->jindF].sdeg[job->gammaF];
    if (dI < 0 || dI >= sI || dF < 0 || dF >= sF)
        return set_error(GAIN_ERR_INVALID_ARG, "components (%d, %d) outside the degeneracies (%d, %d)", dI, dF, sI, sF);
    e->have_amp = false;
    e->have_bnd = false;
    e->ev_up_fresh = false;
    gain_status r;
    if (path == GAIN_PATH_PLAIN_FP64)
        r = e->pieces.size() > 1 ? run_plain_pieces(e, job, dI, dF, stats) : run_plain(e, job, dI, dF, stats);
    else if (path == GAIN_PATH_SPLIT)
        r = run_split(e, job, dI, dF, opts, stats);
    else
        return set_error(GAIN_ERR_INVALID_ARG, "unknown path %d", (int)path);
    e->amp_job = r == GAIN_OK ? job_key(job, dI, dF) : std::vector<int>();
    if (r == GAIN_OK) {   // the run's readers of the eigenvectors are done
        GAIN_CUDA(cudaEventRecord(e->ev_up, e->st));
        e->ev_up_fresh = true;
    }
    return r;
}
}  // namespace

gain_status gain_run_pair(gain_engine e, const gain_pair_job* job, gain_path path, const gain_split_opts* opts,
                          gain_stats* stats) {
    clear_error();
    return run_component(e, job, 0, 0, path, opts, stats);
}

gain_status gain_run_pair_component(gain_engine e, const gain_pair_job* job, int idegI, int idegF, gain_path path,
                                    const gain_split_opts* opts, gain_stats* stats) {
    clear_error();
    GAIN_TRY(run_component(e, job, idegI, idegF, path, opts, stats));
    // keep the amplitudes in the job's component slot (compact rows x cols)
    const std::vector<int> key = job_key(job);
    const size_t n = (size_t)job->nlower * job->nupper;
    const int md = e->maxdeg;
    if (e->deg_job != key) {
        e->deg_job.clear();
        e->deg_filled = 0;
        GAIN_TRY(e->deg_amp.alloc((size_t)md * md * n));
        GAIN_TRY(e->deg_bnd.alloc((size_t)md * md * n));
        e->deg_job = key;
    }
    const int slot = idegI + idegF * md;
    GAIN_CUDA(cudaMemcpy2DAsync(e->deg_amp.p + (size_t)slot * n, sizeof(double) * job->nupper, e->amp.p,
                                sizeof(double) * e->amp_ld, sizeof(double) * job->nupper, job->nlower,
                                cudaMemcpyDeviceToDevice, e->st));
    // the slot's amplitude bounds: the split run's, or zero (the plain path is the FP64 method)
    if (e->have_bnd)
        GAIN_CUDA(cudaMemcpy2DAsync(e->deg_bnd.p + (size_t)slot * n, sizeof(float) * job->nupper, e->ampbnd.p,
                                    sizeof(float) * e->amp_ld, sizeof(float) * job->nupper, job->nlower,
                                    cudaMemcpyDeviceToDevice, e->st));
    else
        GAIN_CUDA(cudaMemsetAsync(e->deg_bnd.p + (size_t)slot * n, 0, sizeof(float) * n, e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    e->deg_filled |= 1u << slot;
    return GAIN_OK;
}

gain_status gain_run_pair_degenerate(gain_engine e, const gain_pair_job* job, const gain_filters* f,
                                     gain_path path, const gain_split_opts* opts, gain_stats* stats) {
    clear_error();
    GAIN_TRY(check_engine(e));
    GAIN_TRY(validate_job(e, job));
    if (!f || !f->sym_degen || f->nsym != e->nsym)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_run_pair_degenerate: filters of %d symmetries needed", e->nsym);
    const int nI = f->sym_degen[job->gammaI], nF = f->sym_degen[job->gammaF];
    if (nI != e->infl[job->jindI].sdeg[job->gammaI] || nF != e->infl[job->jindF].sdeg[job->gammaF])
        return set_error(GAIN_ERR_INVALID_ARG, "sym_degen differs from the expansion tables' degeneracies");
    gain_stats sum;
    memset(&sum, 0, sizeof sum);
    int runs = 0;
    for (int dF = 0; dF < nF; ++dF)      // Output.cpp:78-79 order: idegF outer, idegI inner
        for (int dI = 0; dI < nI; ++dI) {
            if (!gain_degeneracy_filter(f, job->gammaI, job->gammaF, dI, dF)) continue;
            gain_stats one;
            GAIN_TRY(gain_run_pair_component(e, job, dI, dF, path, opts, &one));
            sum.device_ms += one.device_ms;
            sum.refined += one.refined;
            sum.uncertified += one.uncertified;
            sum.uncertified_weak += one.uncertified_weak;
            sum.inexact += one.inexact;
            sum.amp_max = std::max(sum.amp_max, one.amp_max);
            sum.kernel_launches += one.kernel_launches;
            sum.gemm1_ms += one.gemm1_ms;
            sum.gemm2_ms += one.gemm2_ms;
            sum.tensor_flops += one.tensor_flops;
            sum.rows = one.rows;
            sum.cols = one.cols;
            ++runs;
        }
    if (!runs) return set_error(GAIN_ERR_INVALID_ARG, "no component pair passes the degeneracy filter");
    if (stats) *stats = sum;
    return GAIN_OK;
}

gain_status gain_run_plan(gain_engine* engines, int n_engines, const gain_pair_job* jobs, int n_jobs,
                          gain_path path, const gain_split_opts* opts, gain_job_done_fn on_done, void* user,
                          gain_stats* stats) {
    clear_error();
    if (!engines || n_engines <= 0 || n_engines > 64 || (!jobs && n_jobs > 0) || n_jobs < 0)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_run_plan: bad engine or job list");
    for (int i = 0; i < n_engines; ++i) {
        if (!engines[i]) return set_error(GAIN_ERR_INVALID_ARG, "gain_run_plan: engine %d is NULL", i);
        for (int k = 0; k < i; ++k)
            if (engines[k] == engines[i]) return set_error(GAIN_ERR_INVALID_ARG, "gain_run_plan: engine %d repeated", i);
    }
    // largest jobs first (longest-processing-time order): the small ones fill in at the end
    std::vector<int> order(n_jobs);
    for (int j = 0; j < n_jobs; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long long)jobs[a].nlower * jobs[a].nupper > (long long)jobs[b].nlower * jobs[b].nupper;
    });
    std::atomic<int> next{0};
    std::atomic<bool> failed{false};
    std::mutex mu;
    gain_status first_status = GAIN_OK;
    std::string first_error;
    auto worker = [&](gain_engine e) {
        for (;;) {
            if (failed.load()) return;
            const int k = next.fetch_add(1);
            if (k >= n_jobs) return;
            const int j = order[k];
            gain_stats st;
            memset(&st, 0, sizeof st);
            const gain_status r = gain_run_pair(e, &jobs[j], path, opts, &st);
            if (stats) stats[j] = st;
            if (r != GAIN_OK) {
                std::lock_guard<std::mutex> g(mu);
                if (first_status == GAIN_OK) {
                    first_status = r;
                    first_error = "job " + std::to_string(j) + ": " + g_last_error;
                }
                failed.store(true);
            }
            if (on_done) on_done(user, j, e, r);
            if (r != GAIN_OK) return;
        }
    };
    std::vector<std::thread> threads;
    const int nt = std::min(n_engines, std::max(n_jobs, 1));
    for (int i = 1; i < nt; ++i) threads.emplace_back(worker, engines[i]);
    worker(engines[0]);   // the calling thread drives the first engine
    for (auto& t : threads) t.join();
    if (first_status != GAIN_OK) return set_error(first_status, "%s", first_error.c_str());
    return GAIN_OK;
}

gain_status gain_selftest_bounded_wait(gain_engine e, double limit_ms) {
    clear_error();
    GAIN_TRY(check_engine(e));
    if (!(limit_ms > 0.0) || limit_ms > 1000.0)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_selftest_bounded_wait: limit outside (0, 1000] ms");
    GAIN_TRY(e->err.alloc(1));
    GAIN_TRY(e->err.zero(e->st, 1));
    GAIN_CUDA(split::launch_wait_selftest((unsigned long long)(limit_ms * 1e6), e->err.p, e->st));
    int code = 0;
    GAIN_CUDA(cudaMemcpyAsync(&code, e->err.p, sizeof code, cudaMemcpyDeviceToHost, e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    if (code != 0)
        return set_error(GAIN_ERR_TIMEOUT, "bounded device wait gave up after %.3f ms (code %d)", limit_ms, code);
    return GAIN_OK;
}

gain_status gain_pair_amp_device(gain_engine e, const double** amp, int* ld) {
    clear_error();
    if (!e || !amp || !ld) return set_error(GAIN_ERR_INVALID_ARG, "NULL argument");
    if (!e->have_amp) return set_error(GAIN_ERR_NOT_READY, "no completed run");
    *amp = e->amp.p;
    *ld = (int)e->amp_ld;
    return GAIN_OK;
}

gain_status gain_fetch_amp(gain_engine e, double* amp_host) {
    clear_error();
    GAIN_TRY(check_engine(e));
    if (!amp_host) return set_error(GAIN_ERR_INVALID_ARG, "NULL output");
    if (!e->have_amp) return set_error(GAIN_ERR_NOT_READY, "no completed run");
    GAIN_CUDA(cudaMemcpy2DAsync(amp_host, sizeof(double) * e->amp_cols, e->amp.p, sizeof(double) * e->amp_ld,
                                sizeof(double) * e->amp_cols, e->amp_rows, cudaMemcpyDeviceToHost, e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    return GAIN_OK;
}

namespace {
// A pending asynchronous line assembly completes: its copies have landed, n_lines is set and
// the line buffers are free again.
gain_status lines_settle(gain_engine e) {
    if (!e->lines_pending) return GAIN_OK;
    e->lines_pending = false;
    GAIN_CUDA(cudaEventSynchronize(e->ev_lines_d2h));
    if (e->lines_nout) *e->lines_nout = (long long)*(const unsigned long long*)((const char*)e->readback + 96);
    e->lines_nout = nullptr;
    return GAIN_OK;
}

// Line-list membership under THRESH_LINE (Output.cpp:95-96) for split-path amplitudes: the
// lines whose A lies within its certified bound of the threshold are recomputed by the plain
// FP64 path (the reference's method) for every component the line combines, and those
// amplitudes replace the split ones (their bounds become 0) before the line assembly reads
// them.  Energies are on the device (eIdev, eFdev).
constexpr int kThreshCap = 1 << 16;
gain_status thresh_certify(gain_engine e, const gain_line_params* prm, const LineParams& p, const double* amp, long ld) {
    e->thresh_refined = 0;
    if (!(prm->thresh > 0.0)) return GAIN_OK;
    if (p.nslot == 0 && !e->have_bnd) return GAIN_OK;   // the plain path is the FP64 method itself
    const int rows = e->amp_rows, cols = e->amp_cols;
    const size_t n = (size_t)rows * cols;
    const float* bnd = p.nslot == 0 ? e->ampbnd.p : e->deg_bnd.p;
    const long ldb = p.nslot == 0 ? e->amp_ld : cols;
    cudaStream_t st = e->st;
    GAIN_TRY(e->thr_list.alloc(kThreshCap));
    GAIN_TRY(e->thr_cnt.alloc(1));
    GAIN_TRY(e->thr_cnt.zero(st, 1));
    GAIN_CUDA(launch_thresh_flag(rows, cols, amp, ld, bnd, ldb, e->eIdev.p, e->eFdev.p, p, e->thr_list.p,
                                 e->thr_cnt.p, kThreshCap, st));
    unsigned int cnt = 0;
    GAIN_CUDA(cudaMemcpyAsync(&cnt, e->thr_cnt.p, sizeof cnt, cudaMemcpyDeviceToHost, st));
    GAIN_CUDA(cudaStreamSynchronize(st));
    if (cnt == 0) return GAIN_OK;
    if (cnt > (unsigned)kThreshCap)
        return set_error(GAIN_ERR_TOL_NOT_MET, "%u lines lie within their bound of THRESH_LINE (at most %d are "
                         "recomputed)", cnt, kThreshCap);
    std::vector<int2> list(cnt);
    GAIN_CUDA(cudaMemcpy(list.data(), e->thr_list.p, sizeof(int2) * cnt, cudaMemcpyDeviceToHost));
    e->ev_up_fresh = false;   // the FP64 recomputation reads the eigenvectors
    // the job's level lists: job_key = {pair (4), nlower, nupper, dI, dF, lower..., upper...}
    const std::vector<int>& key = e->amp_job;
    if (key.size() < 8 || key[4] != rows || key[5] != cols)
        return set_error(GAIN_ERR_NOT_READY, "THRESH_LINE certification: the amplitudes' job is unknown");
    std::vector<int> R, C;
    for (const int2& rc : list) {
        R.push_back(rc.x);
        C.push_back(rc.y);
    }
    std::sort(R.begin(), R.end());
    R.erase(std::unique(R.begin(), R.end()), R.end());
    std::sort(C.begin(), C.end());
    C.erase(std::unique(C.begin(), C.end()), C.end());
    std::vector<int> lev_lo(R.size()), lev_up(C.size());
    for (size_t i = 0; i < R.size(); ++i) lev_lo[i] = key[8 + R[i]];
    for (size_t i = 0; i < C.size(); ++i) lev_up[i] = key[8 + rows + C[i]];
    GAIN_TRY(e->sub_lower.upload(lev_lo));
    GAIN_TRY(e->sub_upper.upload(lev_up));
    gain_pair_job sj;
    sj.jindI = key[0];
    sj.gammaI = key[1];
    sj.jindF = key[2];
    sj.gammaF = key[3];
    sj.nlower = (int)R.size();
    sj.lower_levels = lev_lo.data();
    sj.nupper = (int)C.size();
    sj.upper_levels = lev_up.data();
    const size_t ns = R.size() * C.size();
    GAIN_TRY(e->sub_amp.alloc(ns));
    // components: the last run's, or every slot the lines combine
    std::vector<std::pair<int, int>> comps;
    std::vector<size_t> base;
    if (p.nslot == 0) {
        comps.push_back({key[6], key[7]});
        base.push_back(0);
    } else {
        for (int q = 0; q < p.nslot; ++q) {
            comps.push_back({p.slot[q] % e->maxdeg, p.slot[q] / e->maxdeg});
            base.push_back((size_t)p.slot[q] * n);
        }
    }
    double* dst = p.nslot == 0 ? e->amp.p : e->deg_amp.p;
    float* dstb = p.nslot == 0 ? e->ampbnd.p : e->deg_bnd.p;
    std::vector<long long> pairs(2 * (size_t)cnt);
    for (size_t q = 0; q < comps.size(); ++q) {
        const int npieces = e->pieces.size() > 1 ? (int)e->pieces.size() : 1;
        for (int pc = 0; pc < npieces; ++pc) {
            if (npieces > 1) GAIN_TRY(load_piece(e, pc));
            double* out = e->sub_amp.p;
            if (pc > 0) {
                GAIN_TRY(e->sub_acc.alloc(ns));
                out = e->sub_acc.p;
            }
            GAIN_TRY(plain_amps(e, &sj, comps[q].first, comps[q].second, e->sub_lower.p, sj.nlower, e->sub_upper.p,
                                sj.nupper, out, nullptr));
            if (pc > 0) GAIN_CUDA(launch_add(e->sub_amp.p, e->sub_acc.p, (long)ns, st));
        }
        for (unsigned int k = 0; k < cnt; ++k) {
            const int r = list[k].x, c = list[k].y;
            const size_t ri = std::lower_bound(R.begin(), R.end(), r) - R.begin();
            const size_t ci = std::lower_bound(C.begin(), C.end(), c) - C.begin();
            pairs[2 * k] = (long long)(base[q] + (size_t)r * (p.nslot == 0 ? (size_t)ld : (size_t)cols) + c);
            pairs[2 * k + 1] = (long long)(ri * C.size() + ci);
        }
        GAIN_TRY(e->sub_patch.upload(pairs));
        GAIN_CUDA(launch_patch((int)cnt, e->sub_patch.p, e->sub_amp.p, dst, dstb, st));
        GAIN_CUDA(cudaStreamSynchronize(st));   // sub_amp and the pair list are reused by the next component
    }
    e->thresh_refined = cnt;
    GAIN_CUDA(cudaEventRecord(e->ev_up, st));
    e->ev_up_fresh = true;
    return GAIN_OK;
}

gain_status pair_lines(gain_engine e, const gain_line_params* prm, const double* energiesI, const double* energiesF,
                       int jI, int jF, double* S, double* A, double* I, unsigned char* keep, long long* n_lines,
                       bool async) {
    GAIN_TRY(check_engine(e));
    GAIN_TRY(lines_settle(e));
    if (!prm || !energiesI || !energiesF || jI < 0 || jF < 0)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_pair_lines: bad argument");
    if (!e->have_amp) return set_error(GAIN_ERR_NOT_READY, "no completed run");
    if (prm->temperature <= 0 || prm->q_part <= 0)
        return set_error(GAIN_ERR_INVALID_ARG, "temperature and partition function must be positive");
    LineParams p = line_params(prm, jI, jF, I != nullptr);
    const double* amp = nullptr;
    long ld = 0;
    GAIN_TRY(line_source(e, prm, p, &amp, &ld));
    const int rows = e->amp_rows, cols = e->amp_cols;
    const size_t n = (size_t)rows * cols;
    cudaStream_t st = e->st;
    GAIN_TRY(e->eIdev.upload(energiesI, rows));
    GAIN_TRY(e->eFdev.upload(energiesF, cols));
    GAIN_TRY(thresh_certify(e, prm, p, amp, ld));
    if (S) GAIN_TRY(e->lineS.alloc(n));
    if (A) GAIN_TRY(e->lineA.alloc(n));
    if (I) GAIN_TRY(e->lineI.alloc(n));
    if (keep) GAIN_TRY(e->lineKeep.alloc(n));
    GAIN_TRY(e->lcnt.alloc(1));
    GAIN_TRY(e->lcnt.zero(st, 1));
    // only the requested outputs are written
    GAIN_CUDA(launch_lines(rows, cols, amp, ld, e->eIdev.p, e->eFdev.p, p, S ? e->lineS.p : nullptr,
                           A ? e->lineA.p : nullptr, I ? e->lineI.p : nullptr, keep ? e->lineKeep.p : nullptr,
                           e->lcnt.p, st));
    if (async) {
        // the copies run on their own stream: the engine's next run (on st, after the line
        // kernel) and its uploads overlap them
        if (!e->readback) GAIN_CUDA(cudaMallocHost(&e->readback, 128));
        GAIN_CUDA(cudaEventRecord(e->ev_lines, st));
        GAIN_CUDA(cudaStreamWaitEvent(e->std2h, e->ev_lines, 0));
        cudaStream_t sd = e->std2h;
        GAIN_CUDA(cudaMemcpyAsync((char*)e->readback + 96, e->lcnt.p, sizeof(unsigned long long),
                                  cudaMemcpyDeviceToHost, sd));
        if (S) GAIN_CUDA(cudaMemcpyAsync(S, e->lineS.p, sizeof(double) * n, cudaMemcpyDeviceToHost, sd));
        if (A) GAIN_CUDA(cudaMemcpyAsync(A, e->lineA.p, sizeof(double) * n, cudaMemcpyDeviceToHost, sd));
        if (I) GAIN_CUDA(cudaMemcpyAsync(I, e->lineI.p, sizeof(double) * n, cudaMemcpyDeviceToHost, sd));
        if (keep) GAIN_CUDA(cudaMemcpyAsync(keep, e->lineKeep.p, n, cudaMemcpyDeviceToHost, sd));
        GAIN_CUDA(cudaEventRecord(e->ev_lines_d2h, sd));
        e->lines_pending = true;
        e->lines_nout = n_lines;
        return GAIN_OK;
    }
    unsigned long long nk = 0;
    GAIN_CUDA(cudaMemcpyAsync(&nk, e->lcnt.p, sizeof nk, cudaMemcpyDeviceToHost, st));
    if (S) GAIN_CUDA(cudaMemcpyAsync(S, e->lineS.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (A) GAIN_CUDA(cudaMemcpyAsync(A, e->lineA.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (I) GAIN_CUDA(cudaMemcpyAsync(I, e->lineI.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (keep) GAIN_CUDA(cudaMemcpyAsync(keep, e->lineKeep.p, n, cudaMemcpyDeviceToHost, st));
    GAIN_CUDA(cudaStreamSynchronize(st));
    if (n_lines) *n_lines = (long long)nk;
    return GAIN_OK;
}
}  // namespace

gain_status gain_pair_lines(gain_engine e, const gain_line_params* prm, const double* energiesI,
                            const double* energiesF, int jI, int jF, double* S, double* A, double* I,
                            unsigned char* keep, long long* n_lines) {
    clear_error();
    return pair_lines(e, prm, energiesI, energiesF, jI, jF, S, A, I, keep, n_lines, false);
}

gain_status gain_pair_lines_async(gain_engine e, const gain_line_params* prm, const double* energiesI,
                                  const double* energiesF, int jI, int jF, double* S, double* A, double* I,
                                  unsigned char* keep, long long* n_lines) {
    clear_error();
    return pair_lines(e, prm, energiesI, energiesF, jI, jF, S, A, I, keep, n_lines, true);
}

gain_status gain_lines_wait(gain_engine e) {
    clear_error();
    GAIN_TRY(check_engine(e));
    return lines_settle(e);
}

gain_status gain_lines_intensity_host(gain_engine e, long long* n_lines) {
    clear_error();
    GAIN_TRY(check_engine(e));
    if (!n_lines) return set_error(GAIN_ERR_INVALID_ARG, "gain_lines_intensity_host: NULL output");
    *n_lines = e->intensity_host;
    return GAIN_OK;
}

gain_status gain_lines_threshold_refined(gain_engine e, long long* n_lines) {
    clear_error();
    GAIN_TRY(check_engine(e));
    if (!n_lines) return set_error(GAIN_ERR_INVALID_ARG, "gain_lines_threshold_refined: NULL output");
    *n_lines = e->thresh_refined;
    return GAIN_OK;
}

namespace {
constexpr int kHardCap = 1 << 20;

// The intensity of Output.cpp:101-102 in line_eval's operation order (every product and
// quotient rounded once; this file is built without floating-point contraction), with this
// host's exp -- the value the reference's own sprintf prints.
double host_intensity(const LineParams& p, double A, double nu, double eI) {
    double t = p.cmcoef * A;
    t = t * p.gnsF;
    t = t * p.two_jF1;
    t = t * std::exp(-p.beta * (eI - p.zpe));
    t = t * (1.0 - std::exp(-p.beta * nu));
    return t / ((nu * nu) * p.q_part);
}

// The text of the last run's lines: lengths, offsets and (into out, when given and large
// enough) the text itself, its device-to-host copy in parts that overlap the formatting of
// the following parts.
gain_status lines_text(gain_engine e, const gain_line_params* prm, const double* energiesI, const double* energiesF,
                       int jI, int jF, int gammaI, int gammaF, int flags, char* out, unsigned long long cap,
                       unsigned long long* text_bytes, long long* n_lines) {
    GAIN_TRY(check_engine(e));
    GAIN_TRY(lines_settle(e));
    if (!prm || !energiesI || !energiesF || jI < 0 || jF < 0 || gammaI < 0 || gammaF < 0 ||
        (flags & ~(GAIN_TEXT_INTENSITY | GAIN_TEXT_AMPLITUDES)))
        return set_error(GAIN_ERR_INVALID_ARG, "gain_pair_lines_text: bad argument");
    if (!e->have_amp) return set_error(GAIN_ERR_NOT_READY, "no completed run");
    if (prm->temperature <= 0 || prm->q_part <= 0)
        return set_error(GAIN_ERR_INVALID_ARG, "temperature and partition function must be positive");
    LineParams lp = line_params(prm, jI, jF, (flags & GAIN_TEXT_INTENSITY) != 0);
    const double* amp = nullptr;
    long ld = 0;
    GAIN_TRY(line_source(e, prm, lp, &amp, &ld));
    e->have_text = false;
    const int rows = e->amp_rows, cols = e->amp_cols;
    const size_t n = (size_t)rows * cols;
    const long nb = text_blocks((long)n);
    cudaStream_t st = e->st;
    GAIN_TRY(e->eIdev.upload(energiesI, rows));
    GAIN_TRY(e->eFdev.upload(energiesF, cols));
    GAIN_TRY(thresh_certify(e, prm, lp, amp, ld));
    GAIN_TRY(e->textLens.alloc(n));
    GAIN_TRY(e->textBlocks.alloc(nb + 3));
    GAIN_TRY(e->textBlocks.zero(st, nb + 3));
    TextArgs t;
    t.rows = rows;
    t.cols = cols;
    t.amp = amp;
    t.ld = ld;
    t.eI = e->eIdev.p;
    t.eF = e->eFdev.p;
    t.p = lp;
    t.levI = e->d_lower.p;
    t.levF = e->d_upper.p;
    t.jI = jI;
    t.jF = jF;
    t.gammaI = gammaI;
    t.gammaF = gammaF;
    t.with_amps = (flags & GAIN_TEXT_AMPLITUDES) != 0;
    t.lens = e->textLens.p;
    t.block_bytes = e->textBlocks.p;
    t.nkeep = e->textBlocks.p + nb + 1;
    t.text = nullptr;
    t.text_size = 0;
    t.hard = nullptr;
    t.nhard = nullptr;
    t.hard_cap = 0;
    t.pow10 = nullptr;
    t.ovr_idx = nullptr;
    t.ovr_val = nullptr;
    t.n_ovr = 0;
    if (lp.with_intensity) {
        if (!e->pow10.p) {
            std::vector<double> pw(601);
            for (int k = -300; k <= 300; ++k) {
                char b[16];
                snprintf(b, sizeof b, "1e%d", k);
                pw[k + 300] = strtod(b, nullptr);
            }
            GAIN_TRY(e->pow10.upload(pw));
        }
        t.pow10 = e->pow10.p;
        GAIN_TRY(e->hardLines.alloc(kHardCap));
        GAIN_TRY(e->hardCount.alloc(1));
        GAIN_TRY(e->hardCount.zero(st, 1));
        t.hard = e->hardLines.p;
        t.nhard = e->hardCount.p;
        t.hard_cap = kHardCap;
    }
    GAIN_CUDA(launch_text_len(t, st));
    std::vector<unsigned long long> offs(nb + 3);   // block offsets, text size, lines, largest block
    unsigned int nhard = 0;
    GAIN_CUDA(cudaMemcpyAsync(offs.data(), e->textBlocks.p, sizeof(unsigned long long) * (nb + 3),
                              cudaMemcpyDeviceToHost, st));
    if (t.nhard) GAIN_CUDA(cudaMemcpyAsync(&nhard, t.nhard, sizeof nhard, cudaMemcpyDeviceToHost, st));
    GAIN_CUDA(cudaStreamSynchronize(st));
    e->intensity_host = 0;
    if (nhard > 0) {
        // Output.cpp:101-102 on the host, with this host's exp, for the lines whose printed
        // intensity the device's exp could change; both passes then print these values
        if (nhard > (unsigned)kHardCap)
            return set_error(GAIN_ERR_UNSUPPORTED, "%u lines need the host's intensity (at most %d)", nhard, kHardCap);
        std::vector<TextArgs::HardLine> hl(nhard);
        GAIN_CUDA(cudaMemcpy(hl.data(), e->hardLines.p, sizeof(TextArgs::HardLine) * nhard, cudaMemcpyDeviceToHost));
        std::sort(hl.begin(), hl.end(), [](const TextArgs::HardLine& a, const TextArgs::HardLine& b) {
            return a.idx < b.idx;
        });
        std::vector<long long> oi(nhard);
        std::vector<double> ov(nhard);
        bool relen = false;
        for (unsigned int k = 0; k < nhard; ++k) {
            oi[k] = hl[k].idx;
            ov[k] = host_intensity(lp, hl[k].A, hl[k].nu, hl[k].eI);
            char b1[64], b2[64];
            relen = relen || snprintf(b1, sizeof b1, "%16.9E", hl[k].I) != snprintf(b2, sizeof b2, "%16.9E", ov[k]);
        }
        GAIN_TRY(e->ovrIdx.upload(oi));
        GAIN_TRY(e->ovrVal.upload(ov));
        t.ovr_idx = e->ovrIdx.p;
        t.ovr_val = e->ovrVal.p;
        t.n_ovr = (int)nhard;
        e->intensity_host = nhard;
        if (relen) {   // a field length changed (an exponent of three digits, say): lengths again
            t.hard = nullptr;
            GAIN_TRY(e->textBlocks.zero(st, nb + 3));
            GAIN_CUDA(launch_text_len(t, st));
            GAIN_CUDA(cudaMemcpyAsync(offs.data(), e->textBlocks.p, sizeof(unsigned long long) * (nb + 3),
                                      cudaMemcpyDeviceToHost, st));
            GAIN_CUDA(cudaStreamSynchronize(st));
        }
    }
    const unsigned long long total = offs[nb], lines = offs[nb + 1], largest = offs[nb + 2];
    if (text_bytes) *text_bytes = total;
    if (n_lines) *n_lines = (long long)lines;
    GAIN_TRY(e->text.alloc(total ? total : 1));
    t.text = e->text.p;
    t.text_size = total;
    const bool copy = out && cap >= total;
    // parts of at least 64 blocks (about 6 MB of text) each, at most 8
    const long nparts = copy ? std::max(1L, std::min(8L, nb / 64)) : 1;
    for (long part = 0; part < nparts; ++part) {
        const long b0 = nb * part / nparts, b1 = nb * (part + 1) / nparts;
        GAIN_CUDA(launch_text_write(t, largest, b0, b1, st));
        if (copy) {
            const unsigned long long o0 = offs[b0], o1 = b1 < nb ? offs[b1] : total;
            GAIN_CUDA(cudaEventRecord(e->ev[8], st));
            GAIN_CUDA(cudaStreamWaitEvent(e->stc, e->ev[8], 0));
            if (o1 > o0) GAIN_CUDA(cudaMemcpyAsync(out + o0, e->text.p + o0, o1 - o0, cudaMemcpyDeviceToHost, e->stc));
        }
    }
    GAIN_CUDA(cudaStreamSynchronize(st));
    if (copy) GAIN_CUDA(cudaStreamSynchronize(e->stc));
    e->text_bytes = total;
    e->have_text = true;
    if (out && !copy)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_pair_lines_text_host: buffer of %llu bytes, text of %llu", cap,
                         total);
    return GAIN_OK;
}
}  // namespace

gain_status gain_pair_lines_text(gain_engine e, const gain_line_params* prm, const double* energiesI,
                                 const double* energiesF, int jI, int jF, int gammaI, int gammaF, int flags,
                                 unsigned long long* text_bytes, long long* n_lines) {
    clear_error();
    return lines_text(e, prm, energiesI, energiesF, jI, jF, gammaI, gammaF, flags, nullptr, 0, text_bytes, n_lines);
}

gain_status gain_pair_lines_text_host(gain_engine e, const gain_line_params* prm, const double* energiesI,
                                      const double* energiesF, int jI, int jF, int gammaI, int gammaF, int flags,
                                      char* out, unsigned long long cap, unsigned long long* text_bytes,
                                      long long* n_lines) {
    clear_error();
    if (!out) return set_error(GAIN_ERR_INVALID_ARG, "gain_pair_lines_text_host: NULL output");
    return lines_text(e, prm, energiesI, energiesF, jI, jF, gammaI, gammaF, flags, out, cap, text_bytes, n_lines);
}

gain_status gain_fetch_lines_text(gain_engine e, char* out, unsigned long long cap) {
    clear_error();
    GAIN_TRY(check_engine(e));
    if (!e->have_text) return set_error(GAIN_ERR_NOT_READY, "no line-list text has been built");
    if (!out || cap < e->text_bytes)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_fetch_lines_text: buffer of %llu bytes, text of %llu",
                         cap, e->text_bytes);
    if (e->text_bytes)
        GAIN_CUDA(cudaMemcpyAsync(out, e->text.p, e->text_bytes, cudaMemcpyDeviceToHost, e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    return GAIN_OK;
}

gain_status gain_lines_text_device(gain_engine e, const char** text, unsigned long long* bytes) {
    clear_error();
    if (!e || !text || !bytes) return set_error(GAIN_ERR_INVALID_ARG, "NULL argument");
    if (!e->have_text) return set_error(GAIN_ERR_NOT_READY, "no line-list text has been built");
    *text = e->text.p;
    *bytes = e->text_bytes;
    return GAIN_OK;
}

gain_status gain_format_values_device(const double* values, long long n, int conv, int width, int prec,
                                      char* out, int stride, int* lens) {
    clear_error();
    if (n < 0 || (n > 0 && (!values || !out || !lens)) || (conv != 'E' && conv != 'f') || prec < 0 ||
        prec > (conv == 'E' ? 17 : 9) || width < 0 || width > 64 || stride <= 0)
        return set_error(GAIN_ERR_INVALID_ARG, "gain_format_values_device: bad argument");
    if (n == 0) return GAIN_OK;
    DevArray<double> v;
    DevArray<char> o;
    DevArray<int> l;
    GAIN_TRY(v.upload(values, (size_t)n));
    GAIN_TRY(o.alloc((size_t)n * stride));
    GAIN_TRY(l.alloc((size_t)n));
    GAIN_CUDA(launch_format_values(n, v.p, conv, width, prec, o.p, stride, l.p, nullptr));
    GAIN_CUDA(cudaMemcpy(out, o.p, (size_t)n * stride, cudaMemcpyDeviceToHost));
    GAIN_CUDA(cudaMemcpy(lens, l.p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
    return GAIN_OK;
}

int gain_format_line(char* buf, size_t cap, double nu, int indexF, int jF, int gammaF, int indexI, int jI,
                     int gammaI, double A, int with_intensity, double intensity, const double* amps, int namp) {
    if (!buf || cap == 0) return 0;
    std::string s;
    char tmp[256];
    snprintf(tmp, sizeof tmp, "%12.6f %8d %4d %4d <- %8d %4d %4d %16.9E ", nu, indexF + 1, jF, gammaF + 1,
             indexI + 1, jI, gammaI + 1, A);
    s += tmp;
    if (with_intensity) {
        snprintf(tmp, sizeof tmp, "%16.9E ", intensity);
        s += tmp;
    }
    if (amps && namp > 0) {
        std::string l;
        for (int i = 0; i < namp; ++i) {
            snprintf(tmp, sizeof tmp, " %16.9E", amps[i]);
            l += tmp;
        }
        s += "[ " + l + " ] ";
    }
    s += " || \n";   // fprintf(output, "%s || \n", buffer), Output.cpp:111
    const size_t n = std::min(cap - 1, s.size());
    memcpy(buf, s.data(), n);
    buf[n] = 0;
    return (int)n;
}

}  // extern "C"

// ====================================================================================
// Grouped plans: every job's split path in two grouped tensor-core launches, captured into a
// CUDA graph (gain_plan_*).
namespace {
constexpr int kPlanStreams = 4;   // concurrent branches of the per-job stages

struct PlanJob {
    std::vector<int> lower, upper;
    gain_pair_job job{};
    std::shared_ptr<PairLayout> L;
    SplitParams p1{}, p2{};
    int beta2 = 0, slices2 = 0;   // the second GEMM's digits when chosen (0: the default rule)
    int B = 0, Bpad = 0, Nu = 0, Nupad = 0, K2 = 0, cap1 = 0, cap2 = 0, klass = 0;
    DevArray<int> d_lower, d_upper, iota;
    DevArray<double> primI, H, Hsym, amp;
    DevArray<float> rowerr, ampbnd;
    DevArray<__nv_bfloat16> Vdig, Hdig, Udig;
    StatsDev Vst, Hst, Ust;
    DevArray<int2> flags1, flags2;
    DevArray<split::Prod> prods1, prods2;
    int nprods1 = 0, nprods2 = 0, fuse1 = 1;
    int uowner = -1;              // a job whose upper digits this one reads (same block, levels, layout)
    int lowner = -1;              // a job whose lower digits this one reads (same block, levels, layout)
    CUtensorMap tmV{}, tmH{}, tmU{};
    const void* vI = nullptr;     // eigenvector and band-digit buffers the graph captured
    const void* vF = nullptr;
    int nlevI = 0, nlevF = 0;     // and the eigenvector blocks' shapes
    const void* band = nullptr;
    gain_status status = GAIN_OK;
};

// Size class of the second GEMM's inner dimension (the autotuner's unit).
int k2_class(int K2) { return K2 <= 2048 ? 0 : K2 <= 8192 ? 1 : K2 <= 16384 ? 2 : 3; }

struct TuneChoice {
    bool pair = false;
    int beta2[4] = {0, 0, 0, 0}, slices2[4] = {0, 0, 0, 0};
};
std::mutex g_tune_mutex;
std::map<std::string, TuneChoice> g_tune_cache;   // plan shape -> choice (this process)
}  // namespace

struct gain_plan_s {
    gain_engine e = nullptr;
    std::vector<std::unique_ptr<PlanJob>> jobs;
    gain_split_opts opts{};
    bool has_opts = false;
    int flags = 0;
    bool pair = false;
    int units = 0;
    DevArray<split::GemmGroup> groups1, groups2;
    DevArray<split::Tile> tiles1, tiles2;
    int ntiles1 = 0, ntiles2 = 0, real1 = 0, real2 = 0;
    int s1max = 1, c1max = 1, s2max = 1, c2max = 1;
    double flops = 0.0;
    // the plan's digit slicings, one launch per slicing kernel: the eigenvectors (before the
    // first GEMM) and H (before the second)
    struct SliceBatch {
        int kernel = 0, n = 0, rows = 0;
        DevArray<split::SliceArgs> args;
        DevArray<int> offs;
    };
    std::vector<SliceBatch> slices1, slices3;
    DevArray<unsigned int> counters;        // [2 * njobs]: GEMM1 / GEMM2 refinement counts
    DevArray<unsigned long long> ull;       // [4 * njobs]: uncertified, -, amp max, uncertified weak
    DevArray<int> err;
    char* rb = nullptr;                     // page-locked readback of counters, ull, err
    cudaStream_t side[kPlanStreams - 1] = {};
    // fork / join order the capture's branches; ev[] are timing events recorded as graph nodes
    // (cudaEventRecordExternal) around the stages
    cudaEvent_t fork = nullptr, join[kPlanStreams - 1] = {}, ev[6] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long dip_version = -1, wig_version = -1, struct_version = -1;
    bool ready = false;
    int captures = 0, graph_nodes = 0, kernel_nodes = 0;
    bool tuned = false;
    double tune_ms = 0.0;
    std::vector<gain_stats> job_stats;

    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        ready = false;
    }
    ~gain_plan_s() {
        if (e) cudaSetDevice(e->device);
        drop_graph();
        for (auto& s : side)
            if (s) cudaStreamDestroy(s);
        if (fork) cudaEventDestroy(fork);
        for (auto& v : join)
            if (v) cudaEventDestroy(v);
        for (auto& v : ev)
            if (v) cudaEventDestroy(v);
        if (rb) cudaFreeHost(rb);
    }
};

namespace {
// Buffers, layout, digit configuration and tensor maps of one job (before any capture).
gain_status plan_prepare_job(gain_plan P, PlanJob& J) {
    gain_engine e = P->e;
    const gain_pair_job* j = &J.job;
    cudaStream_t st = e->st;
    GAIN_TRY(validate_job(e, j));   // the uploads may have changed since the plan was made
    GammaMaps* mI = gamma_maps(e, j->jindI, j->gammaI, 0);
    GammaMaps* mF = gamma_maps(e, j->jindF, j->gammaF, 0);
    if (!mI || !mF) return GAIN_ERR_OOM;
    GAIN_TRY(build_layout(e, j, 0, 0, mI, mF));
    const std::array<int, 6> akey = {j->jindI, j->gammaI, j->jindF, j->gammaF, 0, 0};
    J.L = e->layouts.at(akey);
    PairLayout& L = *J.L;
    const gain_split_opts* opts = P->has_opts ? &P->opts : nullptr;
    J.p1 = gemm1_params(L, opts);
    J.K2 = L.general ? L.ntpad : L.fpad;
    gain_split_opts o2 = P->has_opts ? P->opts : gain_split_opts{};
    if (J.beta2) {
        o2.beta = J.beta2;
        o2.slices = J.slices2;
        o2.kchunks = 0;
    }
    J.p2 = choose_params(J.K2, &o2, 48, 8);
    J.klass = k2_class(J.K2);
    if (!digits_supported(J.p1, J.p2)) return set_error(GAIN_ERR_INVALID_ARG, "unsupported digit configuration");
    GAIN_TRY(layout_band_digits(e, L, J.p1, st));
    const Basis& bI = e->bases[j->jindI];
    const Eig& EI = *e->eig[{j->jindI, j->gammaI}];
    const Eig& EF = *e->eig[{j->jindF, j->gammaF}];
    J.B = j->nlower;
    J.Nu = j->nupper;
    if (L.general && J.B > 65535)
        return set_error(GAIN_ERR_UNSUPPORTED, "plan job with a mixing expansion: at most 65535 lower states");
    const int mstep = P->pair ? 2 * split::BM : split::BM;
    J.Bpad = round_up(J.B, mstep);
    J.Nupad = round_up(J.Nu, split::BN);
    // refinement-list capacity: every entry of a small job (up to 2^20), an eighth of a large
    // one's (at least 2^20, at most the single-pair runs' list)
    auto cap_of = [](long entries) {
        return (int)(entries <= (1L << 20) ? std::max<long>(entries, 1)
                                          : std::min<long>(kMaxFlags, std::max<long>(1L << 20, entries / 8)));
    };
    J.cap1 = cap_of((long)J.Bpad * L.fpad);
    J.cap2 = cap_of((long)J.Bpad * J.Nupad);
    // jobs with the same upper block, upper levels, upper layout and digits share one set of
    // upper digits (the first of them slices it)
    J.uowner = -1;
    for (auto& Q : P->jobs) {
        if (Q.get() == &J) break;
        const PairLayout& QL = *Q->L;
        if (Q->job.jindF == j->jindF && Q->job.gammaF == j->gammaF && Q->upper == J.upper && Q->K2 == J.K2 &&
            Q->p2.beta == J.p2.beta && Q->p2.slices == J.p2.slices && Q->p2.chunks == J.p2.chunks &&
            QL.general == L.general && QL.colposF == L.colposF && QL.f_sym == L.f_sym && QL.nsymF == L.nsymF &&
            Q->uowner < 0) {
            J.uowner = (int)(&Q - &P->jobs[0]);
            break;
        }
    }
    // and likewise jobs with the same lower block, lower levels, lower layout and first-GEMM
    // digits share one set of lower digits (mixing expansions excluded: theirs come from
    // each job's own expansion)
    J.lowner = -1;
    if (!L.general)
        for (auto& Q : P->jobs) {
            if (Q.get() == &J) break;
            const PairLayout& QL = *Q->L;
            if (Q->job.jindI == j->jindI && Q->job.gammaI == j->gammaI && Q->lower == J.lower && Q->Bpad == J.Bpad &&
                Q->p1.beta == J.p1.beta && Q->p1.slices == J.p1.slices && Q->p1.chunks == J.p1.chunks &&
                !QL.general && QL.kpadI == L.kpadI && QL.colposI == L.colposI && QL.i_sym == L.i_sym &&
                Q->lowner < 0) {
                J.lowner = (int)(&Q - &P->jobs[0]);
                break;
            }
        }
    const size_t vdig = J.lowner < 0 ? (size_t)J.p1.slices * J.Bpad * L.kpadI : 0;
    const size_t hdig = (size_t)J.p2.slices * J.Bpad * J.K2;
    const size_t udig = J.uowner < 0 ? (size_t)J.p2.slices * J.Nupad * J.K2 : 0;
    if (J.lowner < 0) {
        GAIN_TRY(J.Vdig.alloc(vdig));
        GAIN_TRY(J.Vdig.zero(st, vdig));
        GAIN_TRY(J.Vst.alloc(J.Bpad, J.p1.chunks, false));
        GAIN_TRY(J.Vst.zero(st, J.Bpad, J.p1.chunks, false));
    } else {   // not this job's: release what an earlier preparation left
        J.Vdig.release();
        J.Vst = StatsDev();
    }
    GAIN_TRY(J.Hdig.alloc(hdig));
    GAIN_TRY(J.Hdig.zero(st, hdig));
    GAIN_TRY(J.Hst.alloc(J.Bpad, J.p2.chunks, true));
    GAIN_TRY(J.Hst.zero(st, J.Bpad, J.p2.chunks, true));
    if (J.uowner < 0) {
        GAIN_TRY(J.Udig.alloc(udig));
        GAIN_TRY(J.Udig.zero(st, udig));
        GAIN_TRY(J.Ust.alloc(J.Nupad, J.p2.chunks, false));
        GAIN_TRY(J.Ust.zero(st, J.Nupad, J.p2.chunks, false));
    } else {   // not this job's: release what an earlier preparation left
        J.Udig.release();
        J.Ust = StatsDev();
    }
    GAIN_TRY(J.H.alloc((size_t)J.Bpad * L.fpad));
    GAIN_TRY(J.rowerr.alloc(J.Bpad));
    GAIN_TRY(J.amp.alloc((size_t)J.Bpad * J.Nupad));
    GAIN_TRY(J.ampbnd.alloc((size_t)J.Bpad * J.Nupad));
    GAIN_TRY(J.flags1.alloc(J.cap1));
    GAIN_TRY(J.flags2.alloc(J.cap2));
    GAIN_TRY(J.d_lower.upload(J.lower));
    GAIN_TRY(J.d_upper.upload(J.upper));
    if (L.general) {
        GAIN_TRY(J.primI.alloc((size_t)J.B * bI.dimen));
        std::vector<int> io(J.B);
        for (int b = 0; b < J.B; ++b) io[b] = b;
        GAIN_TRY(J.iota.upload(io));
        GAIN_TRY(J.Hsym.alloc((size_t)J.Bpad * J.K2));
    }
    J.fuse1 = gemm1_fuse(L, J.p1);
    const std::vector<split::Prod> pr1 = make_prods(J.p1, J.fuse1), pr2 = make_prods(J.p2);
    GAIN_TRY(J.prods1.upload(pr1));
    GAIN_TRY(J.prods2.upload(pr2));
    J.nprods1 = (int)pr1.size();
    J.nprods2 = (int)pr2.size();
    if ((J.lowner < 0 && !split::make_digit_map(&J.tmV, J.Vdig.p, L.kpadI, J.Bpad, J.p1.slices)) ||
        !split::make_digit_map(&J.tmH, J.Hdig.p, J.K2, J.Bpad, J.p2.slices) ||
        (J.uowner < 0 &&
         !split::make_digit_map(&J.tmU, J.Udig.p, J.K2, J.Nupad, J.p2.slices, P->pair ? split::BN / 2 : split::BM)))
        return set_error(GAIN_ERR_CUDA, "cuTensorMapEncodeTiled failed (plan job digits)");
    J.vI = EI.d.p;
    J.vF = EF.d.p;
    J.nlevI = EI.nlevels;
    J.nlevF = EF.nlevels;
    J.band = L.bandDig.p;
    return GAIN_OK;
}

// The slicings `all` grouped by kernel into batches of one launch each (device memory).
gain_status plan_slice_batches(const std::vector<split::SliceArgs>& all, std::vector<gain_plan_s::SliceBatch>& out) {
    out.clear();
    std::map<int, std::vector<split::SliceArgs>> by;
    for (const auto& a : all)
        if (a.nrows > 0) by[split::slice_kernel_of(a)].push_back(a);
    for (auto& kv : by) {
        gain_plan_s::SliceBatch b;
        b.kernel = kv.first;
        b.n = (int)kv.second.size();
        std::vector<int> offs(b.n + 1, 0);
        for (int g = 0; g < b.n; ++g) offs[g + 1] = offs[g] + kv.second[g].nrows;
        b.rows = offs[b.n];
        GAIN_TRY(b.args.upload(kv.second));
        GAIN_TRY(b.offs.upload(offs));
        out.push_back(std::move(b));
    }
    return GAIN_OK;
}

// Every job's slicings: its lower and upper vectors before the first GEMM (only the owner of
// a shared set of lower or upper digits slices it), its H before the second.  Each produces exactly what
// the single-pair run's slicing of the same rows does.
gain_status plan_build_slices(gain_plan P) {
    gain_engine e = P->e;
    std::vector<split::SliceArgs> s1, s3;
    for (auto& Jp : P->jobs) {
        PlanJob& J = *Jp;
        PairLayout& L = *J.L;
        const gain_pair_job* j = &J.job;
        const Eig& EI = *e->eig[{j->jindI, j->gammaI}];
        const Eig& EF = *e->eig[{j->jindF, j->gammaF}];
        const Basis& bI = e->bases[j->jindI];
        if (L.general) {
            s1.push_back(slice_args(J.primI.p, bI.dimen, nullptr, J.B, bI.dimen, nullptr, nullptr, L.kpadI, J.Bpad,
                                    J.Vdig.p, J.p1, J.Vst, false, nullptr, nullptr, L.d_i_sym.p));
            if (J.uowner < 0)
                s1.push_back(slice_args(EF.d.p, EF.nsize, J.d_upper.p, J.Nu, L.nsymF, nullptr, nullptr, J.K2, J.Nupad,
                                        J.Udig.p, J.p2, J.Ust, false, nullptr, nullptr));
        } else {
            if (J.lowner < 0)
                s1.push_back(slice_args(EI.d.p, EI.nsize, J.d_lower.p, J.B, EI.nsize, L.d_colposI.p, &L.colposI,
                                        L.kpadI, J.Bpad, J.Vdig.p, J.p1, J.Vst, false, nullptr, nullptr,
                                        L.d_i_sym.p));
            if (J.uowner < 0)
                s1.push_back(slice_args(EF.d.p, EF.nsize, J.d_upper.p, J.Nu, EF.nsize, L.d_colposF.p, &L.colposF,
                                        L.fpad, J.Nupad, J.Udig.p, J.p2, J.Ust, false, nullptr, nullptr,
                                        L.d_f_sym.p));
        }
        const PlanJob& JL = J.lowner < 0 ? J : *P->jobs[J.lowner];   // the lower digits' owner
        s3.push_back(slice_args(L.general ? J.Hsym.p : J.H.p, J.K2, nullptr, J.B, L.general ? L.nsymF : L.fpad,
                                nullptr, nullptr, J.K2, J.Bpad, J.Hdig.p, J.p2, J.Hst, true, J.rowerr.p,
                                JL.Vst.e.p));
    }
    GAIN_TRY(plan_slice_batches(s1, P->slices1));
    GAIN_TRY(plan_slice_batches(s3, P->slices3));
    return GAIN_OK;
}

// Batch k on stream streams[k % nstreams] (independent outputs: the batches may overlap).
gain_status plan_launch_slices(const std::vector<gain_plan_s::SliceBatch>& batches, const cudaStream_t* streams,
                               int nstreams) {
    for (size_t k = 0; k < batches.size(); ++k) {
        const auto& b = batches[k];
        split::SliceGroups g;
        g.args = b.args.p;
        g.offs = b.offs.p;
        g.n = b.n;
        g.rows = b.rows;
        GAIN_CUDA(split::launch_slice_grouped(g, b.kernel, streams[k % nstreams]));
    }
    return GAIN_OK;
}

// Groups and schedules of both grouped launches.
gain_status plan_build_groups(gain_plan P) {
    gain_engine e = P->e;
    const int mstep = P->pair ? 2 * split::BM : split::BM;
    P->units = P->pair ? e->num_sms / 2 : e->num_sms;
    const int nj = (int)P->jobs.size();
    std::vector<split::GemmGroup> g1(nj), g2(nj);
    std::vector<split::Tile> t1, t2;
    std::vector<double> c1, c2;
    P->s1max = P->c1max = P->s2max = P->c2max = 1;
    P->flops = 0.0;
    const double tol = (P->has_opts && P->opts.tol > 0) ? P->opts.tol : 4.5e-9;
    for (int q = 0; q < nj; ++q) {
        PlanJob& J = *P->jobs[q];
        PairLayout& L = *J.L;
        memset(&g1[q], 0, sizeof g1[q]);
        memset(&g2[q], 0, sizeof g2[q]);
        PlanJob& JL = J.lowner < 0 ? J : *P->jobs[J.lowner];   // the lower digits' owner
        g1[q].tmA = JL.tmV;
        g1[q].tmB = P->pair ? L.tmBandPair : L.tmBand;
        split::GemmArgs& a1 = g1[q].args;
        a1.prods = J.prods1.p;
        a1.nprods = J.nprods1;
        a1.nchunks = J.p1.chunks;
        a1.beta = J.p1.beta;
        a1.slices = J.p1.slices;
        a1.out = J.H.p;
        a1.ldo = L.fpad;
        a1.A = JL.Vst.view(false);
        a1.B = L.bandStats.view(false);
        a1.c_fix = fix_const(J.nprods1);
        a1.c_f64 = (float)((double)(L.W + 64) * std::ldexp(1.0, -53) * 1.01);
        a1.rowerr2 = J.rowerr.p;
        a1.flag_mode = 2;
        a1.tol = (float)tol;
        a1.flags = J.flags1.p;
        a1.nflags = P->counters.p + 2 * q;
        a1.max_flags = J.cap1;
        a1.rows_valid = J.B;
        a1.cols_valid = L.fpad;
        a1.fuse = J.fuse1;
        g2[q].tmA = J.tmH;
        PlanJob& JU = J.uowner < 0 ? J : *P->jobs[J.uowner];   // the upper digits' owner
        g2[q].tmB = JU.tmU;
        split::GemmArgs& a2 = g2[q].args;
        a2.prods = J.prods2.p;
        a2.nprods = J.nprods2;
        a2.nchunks = J.p2.chunks;
        a2.beta = J.p2.beta;
        a2.slices = J.p2.slices;
        a2.out = J.amp.p;
        a2.ldo = J.Nupad;
        a2.A = J.Hst.view(false);
        a2.B = JU.Ust.view(false);
        a2.c_fix = fix_const(J.nprods2);
        a2.c_f64 = (float)((double)((L.general ? L.nsymF : L.nF) + 64) * std::ldexp(1.0, -53) * 1.01);
        a2.absmax = P->ull.p + 4 * q + 2;
        a2.flag_mode = 1;
        a2.tol = (float)tol;
        a2.flags = J.flags2.p;
        a2.nflags = P->counters.p + 2 * q + 1;
        a2.max_flags = J.cap2;
        a2.rows_valid = J.B;
        a2.cols_valid = J.Nu;
        a2.bnd = J.ampbnd.p;
        a2.ldb = J.Nupad;
        P->s1max = std::max(P->s1max, J.p1.slices);
        P->c1max = std::max(P->c1max, J.p1.chunks);
        P->s2max = std::max(P->s2max, J.p2.slices);
        P->c2max = std::max(P->c2max, J.p2.chunks);
        const double tri1 = (double)J.nprods1 / J.p1.chunks, tri2 = (double)J.nprods2 / J.p2.chunks;
        for (auto& fb : L.fblocks)
            for (int n0 = fb.first; n0 < fb.second; n0 += split::BN)
                for (int m0 = 0; m0 < J.Bpad; m0 += mstep) {
                    split::Tile t;
                    memset(&t, 0, sizeof t);
                    t.m0 = m0;
                    t.n0 = n0;
                    t.a_k0 = L.band_k0[n0];
                    t.nkb = L.band_len[n0] / split::BK;
                    t.group = q;
                    t1.push_back(t);
                    c1.push_back(t.nkb * tri1 + 2.0 * J.nprods1);
                    P->flops += 2.0 * mstep * split::BN * split::BK * t.nkb * tri1;
                }
        for (int n0 = 0; n0 < J.Nupad; n0 += split::BN)
            for (int m0 = 0; m0 < J.Bpad; m0 += mstep) {
                split::Tile t;
                memset(&t, 0, sizeof t);
                t.m0 = m0;
                t.n0 = n0;
                t.nkb = J.K2 / split::BK;
                t.group = q;
                t2.push_back(t);
                c2.push_back(t.nkb * tri2 + 2.0 * J.nprods2);
                P->flops += 2.0 * mstep * split::BN * split::BK * t.nkb * tri2;
            }
    }
    // each job's tiles in row groups (concurrent tiles share their operands' digits in L2)
    auto regroup = [&](std::vector<split::Tile>& t, std::vector<double>& c) {
        std::vector<int> idx(t.size());
        for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int)i;
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
            if (t[a].group != t[b].group) return t[a].group < t[b].group;
            return t[a].m0 / (kRowGroup * mstep) < t[b].m0 / (kRowGroup * mstep);
        });
        std::vector<split::Tile> t2s(t.size());
        std::vector<double> c2s(c.size());
        for (size_t i = 0; i < idx.size(); ++i) {
            t2s[i] = t[idx[i]];
            c2s[i] = c[idx[i]];
        }
        t.swap(t2s);
        c.swap(c2s);
    };
    regroup(t1, c1);
    regroup(t2, c2);
    P->real1 = (int)t1.size();
    P->real2 = (int)t2.size();
    const std::vector<split::Tile> s1 = list_schedule(t1, c1, P->units), s2 = list_schedule(t2, c2, P->units);
    P->ntiles1 = (int)s1.size();
    P->ntiles2 = (int)s2.size();
    GAIN_TRY(P->groups1.upload(g1));
    GAIN_TRY(P->groups2.upload(g2));
    GAIN_TRY(P->tiles1.upload(s1));
    GAIN_TRY(P->tiles2.upload(s2));
    return GAIN_OK;
}

// The plan's work on the engine's stream (and its side streams), to be captured.
gain_status plan_enqueue(gain_plan P) {
    gain_engine e = P->e;
    cudaStream_t st = e->st;
    const int nj = (int)P->jobs.size();
    auto stream_of = [&](int q) { return q % kPlanStreams == 0 ? st : P->side[q % kPlanStreams - 1]; };
    auto fork = [&]() -> gain_status {
        GAIN_CUDA(cudaEventRecord(P->fork, st));
        for (auto s : P->side) GAIN_CUDA(cudaStreamWaitEvent(s, P->fork, 0));
        return GAIN_OK;
    };
    auto join = [&]() -> gain_status {
        for (int k = 0; k < kPlanStreams - 1; ++k) {
            GAIN_CUDA(cudaEventRecord(P->join[k], P->side[k]));
            GAIN_CUDA(cudaStreamWaitEvent(st, P->join[k], 0));
        }
        return GAIN_OK;
    };
    GAIN_CUDA(cudaMemsetAsync(P->counters.p, 0, sizeof(unsigned int) * 2 * nj, st));
    GAIN_CUDA(cudaMemsetAsync(P->ull.p, 0, sizeof(unsigned long long) * 4 * nj, st));
    GAIN_CUDA(cudaMemsetAsync(P->err.p, 0, sizeof(int), st));
    GAIN_CUDA(cudaEventRecordWithFlags(P->ev[0], st, cudaEventRecordExternal));
    // ---- stage 1: expansions of mixing lower vectors (per job, on the branches), then the
    // digits of every job's lower and upper eigenvectors (one launch per slicing kernel)
    GAIN_TRY(fork());
    for (int q = 0; q < nj; ++q) {
        PlanJob& J = *P->jobs[q];
        PairLayout& L = *J.L;
        const gain_pair_job* j = &J.job;
        cudaStream_t sq = stream_of(q);
        if (L.general) {
            const Eig& EI = *e->eig[{j->jindI, j->gammaI}];
            const Basis& bI = e->bases[j->jindI];
            Inflation& iI = e->infl[j->jindI];
            GAIN_CUDA(launch_expand_levels(iI.dimen, j->gammaI, iI.maxcoeff, 0, iI.sdeg[j->gammaI], iI.Ntot[j->gammaI],
                                           iI.dijterms.p, iI.dicontr.p, iI.dN[j->gammaI]->p, iI.drepres[j->gammaI]->p,
                                           EI.d.p, EI.nsize, J.d_lower.p, J.primI.p, bI.dimen, J.B, sq));
        }
        GAIN_CUDA(cudaMemsetAsync(J.rowerr.p, 0, sizeof(float) * J.Bpad, sq));
    }
    GAIN_TRY(join());
    cudaStream_t streams[kPlanStreams];
    for (int k = 0; k < kPlanStreams; ++k) streams[k] = stream_of(k);
    GAIN_TRY(fork());
    GAIN_TRY(plan_launch_slices(P->slices1, streams, kPlanStreams));
    GAIN_TRY(join());
    // ---- stage 2: the first GEMM of every job, one grouped launch
    split::GemmArgs ga;
    memset(&ga, 0, sizeof ga);
    ga.err = P->err.p;
    ga.groups = P->groups1.p;
    ga.tiles = P->tiles1.p;
    ga.ntiles = P->ntiles1;
    GAIN_CUDA(cudaEventRecordWithFlags(P->ev[1], st, cudaEventRecordExternal));
    GAIN_CUDA(split::launch_gemm_grouped(ga, P->units, P->s1max, P->c1max, st, P->pair));
    GAIN_CUDA(cudaEventRecordWithFlags(P->ev[2], st, cudaEventRecordExternal));
    // ---- stage 3: FP64 refinement of H, contraction (mixing expansions), digits of H
    GAIN_TRY(fork());
    for (int q = 0; q < nj; ++q) {
        PlanJob& J = *P->jobs[q];
        PairLayout& L = *J.L;
        const gain_pair_job* j = &J.job;
        cudaStream_t sq = stream_of(q);
        const Eig& EI = *e->eig[{j->jindI, j->gammaI}];
        const Basis& bI = e->bases[j->jindI];
        split::RefineHArgs rh;
        rh.flags = J.flags1.p;
        rh.nflags = P->counters.p + 2 * q;
        rh.max_flags = J.cap1;
        rh.vecs = L.general ? J.primI.p : EI.d.p;
        rh.nsize = L.general ? bI.dimen : EI.nsize;
        rh.row_level = L.general ? J.iota.p : J.d_lower.p;
        rh.i_sym = L.d_i_sym.p;
        rh.band_k0 = L.d_band_k0.p;
        rh.band_len = L.d_band_len.p;
        rh.band = L.band.p;
        rh.W = L.W;
        rh.H = J.H.p;
        rh.ldh = L.fpad;
        rh.eA = (J.lowner < 0 ? J : *P->jobs[J.lowner]).Vst.e.p;
        rh.rowerr2 = J.rowerr.p;
        GAIN_CUDA(split::launch_refine_h(rh, std::min(2 * e->num_sms, std::max(1, J.cap1 / 8)), sq));
        if (L.general) {
            GAIN_CUDA(launch_contract_rowerr(J.B, J.H.p, L.fpad, L.fpad, J.rowerr.p, J.Vst.e.p, L.sigmaF, L.gamF, sq));
            GAIN_CUDA(launch_contract(L.nsymF, L.d_cF_ptr.p, L.d_cF_col.p, L.d_cF_val.p, J.H.p, L.fpad, J.Hsym.p, J.K2,
                                      J.B, sq));
        }
    }
    GAIN_TRY(join());
    GAIN_TRY(fork());
    GAIN_TRY(plan_launch_slices(P->slices3, streams, kPlanStreams));   // every job's H digits
    GAIN_TRY(join());
    // ---- stage 4: the second GEMM of every job, one grouped launch
    ga.groups = P->groups2.p;
    ga.tiles = P->tiles2.p;
    ga.ntiles = P->ntiles2;
    GAIN_CUDA(cudaEventRecordWithFlags(P->ev[3], st, cudaEventRecordExternal));
    GAIN_CUDA(split::launch_gemm_grouped(ga, P->units, P->s2max, P->c2max, st, P->pair));
    GAIN_CUDA(cudaEventRecordWithFlags(P->ev[4], st, cudaEventRecordExternal));
    // ---- stage 5: FP64 refinement of the amplitudes
    GAIN_TRY(fork());
    for (int q = 0; q < nj; ++q) {
        PlanJob& J = *P->jobs[q];
        PairLayout& L = *J.L;
        const gain_pair_job* j = &J.job;
        cudaStream_t sq = stream_of(q);
        const Eig& EF = *e->eig[{j->jindF, j->gammaF}];
        split::RefineAmpArgs ra;
        ra.flags = J.flags2.p;
        ra.nflags = P->counters.p + 2 * q + 1;
        ra.max_flags = J.cap2;
        ra.U = EF.d.p;
        ra.nsize = EF.nsize;
        ra.col_level = J.d_upper.p;
        ra.colpos = L.general ? L.d_ident.p : L.d_colposF.p;
        ra.H = L.general ? J.Hsym.p : J.H.p;
        ra.ldh = J.K2;
        ra.h_inerr = J.Hst.inerr.p;
        ra.eH = J.Hst.e.p;
        ra.amp = J.amp.p;
        ra.lda = J.Nupad;
        ra.bnd = J.ampbnd.p;
        ra.ldb = J.Nupad;
        ra.tol = (P->has_opts && P->opts.tol > 0) ? P->opts.tol : 4.5e-9;
        ra.absmax = P->ull.p + 4 * q + 2;
        ra.amp_floor = std::sqrt((P->has_opts && P->opts.s_floor > 0) ? P->opts.s_floor : 1e-10);
        ra.uncertified = P->ull.p + 4 * q;
        ra.uncertified_weak = P->ull.p + 4 * q + 3;
        GAIN_CUDA(split::launch_refine_amp(ra, std::min(4 * e->num_sms, std::max(1, J.cap2 / 8)), sq));
    }
    GAIN_TRY(join());
    GAIN_CUDA(cudaEventRecordWithFlags(P->ev[5], st, cudaEventRecordExternal));
    GAIN_CUDA(cudaMemcpyAsync(P->rb, P->counters.p, sizeof(unsigned int) * 2 * nj, cudaMemcpyDeviceToHost, st));
    GAIN_CUDA(cudaMemcpyAsync(P->rb + 8 * (size_t)nj, P->ull.p, sizeof(unsigned long long) * 4 * nj,
                              cudaMemcpyDeviceToHost, st));
    GAIN_CUDA(cudaMemcpyAsync(P->rb + 40 * (size_t)nj, P->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    return GAIN_OK;
}

// Prepare every job, build the grouped launches and capture the graph.
gain_status plan_build(gain_plan P) {
    gain_engine e = P->e;
    P->drop_graph();
    const int nj = (int)P->jobs.size();
    for (auto& J : P->jobs) GAIN_TRY(plan_prepare_job(P, *J));
    GAIN_TRY(P->counters.alloc(2 * nj));
    GAIN_TRY(P->ull.alloc(4 * nj));
    GAIN_TRY(P->err.alloc(1));
    GAIN_TRY(plan_build_groups(P));
    GAIN_TRY(plan_build_slices(P));
    if (!P->rb) GAIN_CUDA(cudaMallocHost(&P->rb, 40 * (size_t)nj + 64));
    GAIN_CUDA(split::prepare_device());   // kernel attributes are set outside the capture
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    GAIN_CUDA(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
    const gain_status s = plan_enqueue(P);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(e->st, &g);
    if (s != GAIN_OK) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();
        return s;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "capturing the plan");
    P->graph = g;
    GAIN_CUDA(cudaGraphInstantiate(&P->exec, P->graph, 0));
    size_t nodes = 0;
    GAIN_CUDA(cudaGraphGetNodes(P->graph, nullptr, &nodes));
    std::vector<cudaGraphNode_t> nv(nodes);
    GAIN_CUDA(cudaGraphGetNodes(P->graph, nv.data(), &nodes));
    int kern = 0;
    for (auto n : nv) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(n, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kern;
    }
    P->graph_nodes = (int)nodes;
    P->kernel_nodes = kern;
    ++P->captures;
    P->dip_version = e->dip_version;
    P->wig_version = e->wig_version;
    P->struct_version = e->struct_version;
    P->ready = true;
    return GAIN_OK;
}

// The plan's inputs still where the graph read them?
bool plan_current(gain_plan P) {
    gain_engine e = P->e;
    if (!P->ready || P->dip_version != e->dip_version || P->wig_version != e->wig_version ||
        P->struct_version != e->struct_version)
        return false;
    for (auto& J : P->jobs) {
        const gain_pair_job* j = &J->job;
        auto iI = e->eig.find({j->jindI, j->gammaI});
        auto iF = e->eig.find({j->jindF, j->gammaF});
        if (iI == e->eig.end() || iF == e->eig.end()) return false;
        if (iI->second->d.p != J->vI || iF->second->d.p != J->vF || J->L->bandDig.p != J->band) return false;
        if (iI->second->nlevels != J->nlevI || iF->second->nlevels != J->nlevF) return false;
        if (J->L->beta1 != J->p1.beta || J->L->s1 != J->p1.slices || J->L->c1 != J->p1.chunks) return false;
    }
    return true;
}

// One replay: device time, per-job counters and statuses.
gain_status plan_replay(gain_plan P, double* ms_out) {
    gain_engine e = P->e;
    cudaStream_t st = e->st;
    if (!plan_current(P)) GAIN_TRY(plan_build(P));
    for (auto& J : P->jobs) {   // asynchronous eigenvector uploads land before the replay
        const gain_pair_job* j = &J->job;
        const Eig& EI = *e->eig[{j->jindI, j->gammaI}];
        const Eig& EF = *e->eig[{j->jindF, j->gammaF}];
        if (EI.ready) GAIN_CUDA(cudaStreamWaitEvent(st, EI.ready, 0));
        if (EF.ready) GAIN_CUDA(cudaStreamWaitEvent(st, EF.ready, 0));
    }
    e->ev_up_fresh = false;
    GAIN_CUDA(cudaGraphLaunch(P->exec, st));
    GAIN_CUDA(cudaEventRecord(e->ev_up, st));
    GAIN_CUDA(cudaStreamSynchronize(st));
    e->ev_up_fresh = true;
    float ms = 0.f;
    GAIN_CUDA(cudaEventElapsedTime(&ms, P->ev[0], P->ev[5]));
    if (ms_out) *ms_out = ms;
    const int nj = (int)P->jobs.size();
    const unsigned int* cnt = (const unsigned int*)P->rb;
    const unsigned long long* unc = (const unsigned long long*)(P->rb + 8 * (size_t)nj);
    int errw = 0;
    memcpy(&errw, P->rb + 40 * (size_t)nj, sizeof errw);
    P->job_stats.assign(nj, gain_stats{});
    gain_status first = GAIN_OK;
    for (int q = 0; q < nj; ++q) {
        PlanJob& J = *P->jobs[q];
        gain_stats& s = P->job_stats[q];
        memset(&s, 0, sizeof s);
        s.rows = J.B;
        s.cols = J.Nu;
        s.refined = (long long)std::min<unsigned>(cnt[2 * q], J.cap1) + std::min<unsigned>(cnt[2 * q + 1], J.cap2);
        s.inexact = cnt[2 * q];
        s.uncertified = (long long)unc[4 * q];
        s.uncertified_weak = (long long)unc[4 * q + 3];
        s.amp_max = __builtin_bit_cast(double, unc[4 * q + 2]);
        s.beta1 = J.p1.beta;
        s.slices1 = J.p1.slices;
        s.chunks1 = J.p1.chunks;
        s.beta2 = J.p2.beta;
        s.slices2 = J.p2.slices;
        s.chunks2 = J.p2.chunks;
        s.products1 = J.nprods1;
        s.products2 = J.nprods2;
        J.status = GAIN_OK;
        if (errw != 0) J.status = GAIN_ERR_TIMEOUT;
        else if (cnt[2 * q] > (unsigned)J.cap1 || cnt[2 * q + 1] > (unsigned)J.cap2) J.status = GAIN_ERR_TOL_NOT_MET;
        if (J.status != GAIN_OK && first == GAIN_OK) {
            first = J.status;
            if (errw != 0)
                set_error(GAIN_ERR_TIMEOUT, "a bounded device wait of the grouped GEMM gave up (code %d)", errw);
            else
                set_error(GAIN_ERR_TOL_NOT_MET, "plan job %d: more entries need FP64 refinement than its list holds", q);
        }
    }
    return first;
}

std::string plan_shape_key(gain_plan P) {
    std::string k;
    char buf[96];
    for (auto& J : P->jobs) {
        snprintf(buf, sizeof buf, "%d,%d,%d,%d,%d,%d;", J->job.jindI, J->job.gammaI, J->job.jindF, J->job.gammaF,
                 J->job.nlower, J->job.nupper);
        k += buf;
    }
    snprintf(buf, sizeof buf, "|%d|%.3g", P->has_opts ? P->opts.beta * 100 + P->opts.slices : 0,
             P->has_opts ? P->opts.tol : 0.0);
    return k + buf;
}

void plan_apply(gain_plan P, const TuneChoice& c) {
    P->pair = c.pair;
    for (auto& J : P->jobs) {
        const int k = k2_class(J->L ? (J->L->general ? J->L->ntpad : J->L->fpad) : J->K2);
        J->beta2 = c.beta2[k];
        J->slices2 = c.slices2[k];
    }
}

// The autotuner: the plan's own replays time each candidate (the best of two replays after
// one warm-up); a candidate whose replay fails (a refinement list overflowed) is dropped.
// First the tile shape with the default digits, then, one size class at a time, the 7-bit x 7
// digits of the second GEMM against the default 8-bit x 6.
gain_status plan_autotune(gain_plan P, TuneChoice* out) {
    const auto t0 = std::chrono::steady_clock::now();
    auto time_of = [&](const TuneChoice& c, double* best) -> gain_status {
        plan_apply(P, c);
        GAIN_TRY(plan_build(P));
        *best = 1e300;
        for (int r = 0; r < 3; ++r) {
            double ms = 0;
            const gain_status s = plan_replay(P, &ms);
            if (s != GAIN_OK) return s;
            if (r > 0) *best = std::min(*best, ms);
        }
        return GAIN_OK;
    };
    TuneChoice best_c;
    double best = 1e300;
    bool any_pairable = false;
    for (auto& J : P->jobs) any_pairable = any_pairable || J->job.nlower > split::BM;
    for (int pr = 0; pr < (any_pairable ? 2 : 1); ++pr) {
        TuneChoice c;
        c.pair = pr == 1;
        double ms;
        if (time_of(c, &ms) == GAIN_OK && ms < best) {
            best = ms;
            best_c = c;
        }
    }
    if (best >= 1e300) return set_error(GAIN_ERR_TOL_NOT_MET, "autotuner: no candidate configuration ran");
    bool present[4] = {false, false, false, false};
    for (auto& J : P->jobs) present[k2_class(J->K2)] = true;
    for (int k = 0; k < 4; ++k) {
        if (!present[k]) continue;
        TuneChoice c = best_c;
        c.beta2[k] = 7;
        c.slices2[k] = 7;
        double ms;
        if (time_of(c, &ms) == GAIN_OK && ms < 0.99 * best) {
            best = ms;
            best_c = c;
        }
    }
    clear_error();
    *out = best_c;
    P->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GAIN_OK;
}
}  // namespace

gain_status gain_plan_create(gain_engine e, const gain_pair_job* jobs, int n_jobs, const gain_split_opts* opts,
                             int flags, gain_plan* out) {
    clear_error();
    if (!out) return set_error(GAIN_ERR_INVALID_ARG, "gain_plan_create: NULL output");
    *out = nullptr;
    GAIN_TRY(check_engine(e));
    if (!jobs || n_jobs <= 0 || (flags & ~GAIN_PLAN_AUTOTUNE))
        return set_error(GAIN_ERR_INVALID_ARG, "gain_plan_create: bad job list or flags");
    if (e->pieces.size() > 1)
        return set_error(GAIN_ERR_UNSUPPORTED, "plans take a single dipole piece (gain_upload_dipole)");
    std::unique_ptr<gain_plan_s> P(new gain_plan_s());
    P->e = e;
    P->flags = flags;
    if (opts) {
        P->opts = *opts;
        P->has_opts = true;
    }
    for (int q = 0; q < n_jobs; ++q) {
        GAIN_TRY(validate_job(e, &jobs[q]));
        const int sI = e->infl[jobs[q].jindI].sdeg[jobs[q].gammaI], sF = e->infl[jobs[q].jindF].sdeg[jobs[q].gammaF];
        if (sI != 1 || sF != 1)
            return set_error(GAIN_ERR_UNSUPPORTED, "plan job %d: degenerate symmetries run per component pair", q);
        std::unique_ptr<PlanJob> J(new PlanJob());
        J->lower.assign(jobs[q].lower_levels, jobs[q].lower_levels + jobs[q].nlower);
        J->upper.assign(jobs[q].upper_levels, jobs[q].upper_levels + jobs[q].nupper);
        J->job = jobs[q];
        J->job.lower_levels = J->lower.data();
        J->job.upper_levels = J->upper.data();
        P->jobs.push_back(std::move(J));
    }
    for (auto& s : P->side) GAIN_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    GAIN_CUDA(cudaEventCreateWithFlags(&P->fork, cudaEventDisableTiming));
    for (auto& v : P->join) GAIN_CUDA(cudaEventCreateWithFlags(&v, cudaEventDisableTiming));
    for (auto& v : P->ev) GAIN_CUDA(cudaEventCreate(&v));
    // default configuration: CTA pairs when any job fills more than one 128-row block
    TuneChoice c;
    for (auto& J : P->jobs) c.pair = c.pair || J->job.nlower > split::BM;
    if (const char* pe = getenv("GAINLS_GEMM_PAIR")) c.pair = c.pair && pe[0] != '0';
    if (flags & GAIN_PLAN_AUTOTUNE) {
        const std::string key = plan_shape_key(P.get());
        bool hit = false;
        {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end()) {
                c = it->second;
                hit = true;
            }
        }
        if (!hit) {
            plan_apply(P.get(), c);
            GAIN_TRY(plan_build(P.get()));   // layouts and sizes for the size classes
            GAIN_TRY(plan_autotune(P.get(), &c));
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            g_tune_cache[key] = c;
        }
        P->tuned = true;
    }
    plan_apply(P.get(), c);
    GAIN_TRY(plan_build(P.get()));
    *out = P.release();
    return GAIN_OK;
}

gain_status gain_plan_run(gain_plan P, gain_stats* job_stats, gain_plan_stats* stats) {
    clear_error();
    if (!P) return set_error(GAIN_ERR_INVALID_ARG, "plan is NULL");
    GAIN_TRY(check_engine(P->e));
    double ms = 0.0;
    const gain_status s = plan_replay(P, &ms);
    const int nj = (int)P->jobs.size();
    if (job_stats && (int)P->job_stats.size() == nj)
        for (int q = 0; q < nj; ++q) job_stats[q] = P->job_stats[q];
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->device_ms = ms;
        float g1 = 0.f, g2 = 0.f;
        cudaEventElapsedTime(&g1, P->ev[1], P->ev[2]);
        cudaEventElapsedTime(&g2, P->ev[3], P->ev[4]);
        stats->gemm1_ms = g1;
        stats->gemm2_ms = g2;
        float d1 = 0.f, d3 = 0.f, d5 = 0.f;
        cudaEventElapsedTime(&d1, P->ev[0], P->ev[1]);
        cudaEventElapsedTime(&d3, P->ev[2], P->ev[3]);
        cudaEventElapsedTime(&d5, P->ev[4], P->ev[5]);
        stats->digits_ms = d1;
        stats->middle_ms = d3;
        stats->refine_ms = d5;
        for (auto& J : P->jobs) {
            stats->shared_lower += J->lowner >= 0;
            stats->shared_upper += J->uowner >= 0;
        }
        stats->jobs = nj;
        for (int q = 0; q < nj && q < (int)P->job_stats.size(); ++q) {
            stats->transitions += P->job_stats[q].rows * P->job_stats[q].cols;
            stats->refined += P->job_stats[q].refined;
            stats->uncertified += P->job_stats[q].uncertified;
            stats->failed_jobs += P->jobs[q]->status != GAIN_OK;
            const int k = P->jobs[q]->klass;
            stats->beta2[k] = P->jobs[q]->p2.beta;
            stats->slices2[k] = P->jobs[q]->p2.slices;
        }
        stats->graph_nodes = P->graph_nodes;
        stats->kernel_launches = P->kernel_nodes;
        stats->gemm1_tiles = P->real1;
        stats->gemm2_tiles = P->real2;
        stats->units = P->units;
        stats->pair = P->pair ? 1 : 0;
        stats->captures = P->captures;
        stats->tuned = P->tuned ? 1 : 0;
        stats->tune_ms = P->tune_ms;
        stats->tensor_flops = P->flops;
    }
    return s;
}

gain_status gain_plan_amp_device(gain_plan P, int job, const double** amp, int* ld) {
    clear_error();
    if (!P || !amp || !ld) return set_error(GAIN_ERR_INVALID_ARG, "gain_plan_amp_device: NULL argument");
    if (job < 0 || job >= (int)P->jobs.size()) return set_error(GAIN_ERR_INVALID_ARG, "job %d out of range", job);
    if (P->job_stats.empty() || P->jobs[job]->status != GAIN_OK)
        return set_error(GAIN_ERR_NOT_READY, "job %d has no completed run", job);
    *amp = P->jobs[job]->amp.p;
    *ld = P->jobs[job]->Nupad;
    return GAIN_OK;
}

gain_status gain_plan_select(gain_plan P, int job) {
    clear_error();
    if (!P) return set_error(GAIN_ERR_INVALID_ARG, "plan is NULL");
    GAIN_TRY(check_engine(P->e));
    if (job < 0 || job >= (int)P->jobs.size()) return set_error(GAIN_ERR_INVALID_ARG, "job %d out of range", job);
    PlanJob& J = *P->jobs[job];
    if (P->job_stats.empty() || J.status != GAIN_OK) return set_error(GAIN_ERR_NOT_READY, "job %d has no completed run", job);
    gain_engine e = P->e;
    GAIN_TRY(lines_settle(e));
    const size_t n = (size_t)J.Bpad * J.Nupad;
    GAIN_TRY(e->amp.alloc(n));
    GAIN_TRY(e->ampbnd.alloc(n));
    GAIN_CUDA(cudaMemcpyAsync(e->amp.p, J.amp.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, e->st));
    GAIN_CUDA(cudaMemcpyAsync(e->ampbnd.p, J.ampbnd.p, sizeof(float) * n, cudaMemcpyDeviceToDevice, e->st));
    GAIN_TRY(e->d_lower.alloc(J.B));
    GAIN_TRY(e->d_upper.alloc(J.Nu));
    GAIN_CUDA(cudaMemcpyAsync(e->d_lower.p, J.d_lower.p, sizeof(int) * J.B, cudaMemcpyDeviceToDevice, e->st));
    GAIN_CUDA(cudaMemcpyAsync(e->d_upper.p, J.d_upper.p, sizeof(int) * J.Nu, cudaMemcpyDeviceToDevice, e->st));
    GAIN_CUDA(cudaStreamSynchronize(e->st));
    e->amp_rows = J.B;
    e->amp_cols = J.Nu;
    e->amp_ld = J.Nupad;
    e->amp_job = job_key(&J.job, 0, 0);
    e->have_amp = true;
    e->have_bnd = true;
    return GAIN_OK;
}

gain_status gain_plan_destroy(gain_plan P) {
    clear_error();
    delete P;
    return GAIN_OK;
}
