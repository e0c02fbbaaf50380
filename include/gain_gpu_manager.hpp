// gain_gpu_manager.hpp -- drop-in host mirror of GAIN-MPI's GpuManager over the C ABI.
//
// The method set, argument meaning and call order of BaseClasses/GpuManager.h:135-173, so a
// main.cpp-style driver (main.cpp:172-336) keeps its call sites.  Per-transition calls run
// the library's kernel-level drop-ins (gain_expand, gain_hls_kblock, gain_dot) on device
// buffers this class owns, in the reference's order; ExecuteBlockPair runs a whole
// (J'',Gamma'') -> (J',Gamma') block pair through the batched engine instead.
//
// Differences from the reference, on purpose:
//  * errors come back as gain_status / gain::Error exceptions instead of MPI_Abort;
//  * one device stream per OpenMP thread slot, created here (the reference never creates
//    correlate_half_ls_stream, BaseClasses/GpuManager.cpp:349-350);
//  * the 3j table is exact (gain_threej_table).
// Header-only; link with libgainls.so and the CUDA runtime.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "gain_ls.h"

namespace gain {

struct Error : std::runtime_error {
    gain_status status;
    Error(gain_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(gain_status s) {
    if (s != GAIN_OK) throw Error(s, std::string(gain_status_string(s)) + ": " + gain_last_error_string());
}
inline void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(GAIN_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

class GpuManager {
   public:
    // GpuManager(int pgpu_id, int nprocs, bool rotsym), BaseClasses/GpuManager.cpp:69
    GpuManager(int gpu_id, int nprocs, bool rotsym = false) : gpu_id_(gpu_id), nprocs_(nprocs), rotsym_(rotsym) {}
    ~GpuManager() { release(); }
    GpuManager(const GpuManager&) = delete;
    GpuManager& operator=(const GpuManager&) = delete;

    // BaseClasses/GpuManager.cpp:127-213
    void InitializeAndTransferConstants(int jmax, int sym_repres, int pmax_degen) {
        check_cuda(cudaSetDevice(gpu_id_), "cudaSetDevice");
        jmax_ = jmax;
        nsym_ = sym_repres;
        maxdeg_ = pmax_degen;
        std::vector<double> t((size_t)(jmax + 1) * (jmax + 1) * 9);
        check(gain_threej_table(jmax, t.data()));
        threej_ = upload(t.data(), t.size());
        check(gain_engine_create(gpu_id_, jmax, sym_repres, pmax_degen, &engine_));
        for (int i = 0; i < nprocs_; ++i) {
            cudaStream_t s;
            check_cuda(cudaStreamCreate(&s), "cudaStreamCreate");
            dot_stream_.push_back(s);
        }
    }

    // BaseClasses/GpuManager.cpp:215-265; BasisSetT provides the reference BasisSet getters
    template <class BasisSetT>
    void TransferBasisSet(BasisSetT* b) {
        TransferBasisSet(b->GetJval(), b->GetDimensions(), b->GetK(), b->GetKTau(), b->GetVibIndex(),
                         b->GetKBlock(), b->GetKStart());
    }
    void TransferBasisSet(int J, int dimen, const int* K, const int* ktau, const int* vib, const int* kblock,
                          const int* kstart) {
        const int jind = (int)bases_.size();
        check(gain_upload_basis(engine_, jind, J, dimen, K, ktau, vib, kblock, kstart));
        Basis b;
        b.J = J;
        b.dimen = dimen;
        std::vector<int> tau(ktau, ktau + dimen);
        for (auto& t : tau) t &= 1;
        b.tau = upload(tau.data(), tau.size());
        b.K = upload(K, dimen);          // rotsym form: degeneracy index
        b.lev = upload(ktau, dimen);     // rotsym form: rotational level index
        b.vib = upload(vib, dimen);
        b.kblock = upload(kblock, J + 1);
        b.host_kblock.assign(kblock, kblock + J + 1);
        b.kstart.assign(kstart, kstart + J + 1);
        bases_.push_back(b);
    }

    // BaseClasses/GpuManager.cpp:381-422 (same argument list)
    void TransferInflation(int* icontr, int* ijterm, int dimen, int maxsymcoeffs, int matsize,
                           std::vector<double*> repres, std::vector<int*> N, std::vector<int> Ntot,
                           std::vector<int> sym_degen) {
        const int jind = (int)infl_.size();
        std::vector<const int*> Np(N.begin(), N.end());
        std::vector<const double*> Rp(repres.begin(), repres.end());
        check(gain_upload_inflation(engine_, jind, icontr, ijterm, dimen, maxsymcoeffs, matsize, Np.data(),
                                    Rp.data(), Ntot.data(), sym_degen.data()));
        Inflation f;
        f.maxcoeff = maxsymcoeffs;
        f.ijterms = upload(ijterm, (size_t)maxsymcoeffs * nsym_);
        f.icontr = upload(icontr, (size_t)2 * dimen);
        for (int g = 0; g < nsym_; ++g) {
            f.N.push_back(upload(N[g], maxsymcoeffs));
            f.repres.push_back(upload(repres[g], (size_t)Ntot[g] * sym_degen[g] * matsize));
        }
        f.Ntot = Ntot;
        f.sdeg = sym_degen;
        infl_.push_back(f);
    }

    // BaseClasses/GpuManager.cpp:499-526; DipoleT provides the reference Dipole getters
    template <class DipoleT>
    void TransferDipole(DipoleT* d, int block) {
        TransferDipole(d->GetDipolePiece(block), (int)d->GetMaxContracts(), d->GetDipoleStart(block),
                       d->GetDipoleEnd(block), d->GetDipoleNcontr(block));
        current_block_ = block;
        switch_piece_ = [d](int b, const double** piece, int* N, int* s, int* e, int* n) {
            *piece = d->GetDipolePiece(b);
            *N = (int)d->GetMaxContracts();
            *s = d->GetDipoleStart(b);
            *e = d->GetDipoleEnd(b);
            *n = d->GetDipoleNcontr(b);
        };
    }
    // :481-496: the device takes another block of the dipole given to TransferDipole
    void SwitchDipoleBlock(int block) {
        if (!switch_piece_) throw std::runtime_error("SwitchDipoleBlock before TransferDipole(Dipole*, block)");
        const double* piece;
        int N, s, e, n;
        switch_piece_(block, &piece, &N, &s, &e, &n);
        TransferDipole(piece, N, s, e, n);
        current_block_ = block;
    }
    // For ExecuteBlockPair: every block of the dipole at once, kept in host memory; the engine
    // loops over them per run (gain_upload_dipole_pieces).  The pieces must outlive the runs.
    template <class DipoleT>
    void TransferDipolePieces(DipoleT* d) {
        std::vector<const double*> p;
        std::vector<int> s, e;
        for (int b = 0; b < d->GetNumBlocks(); ++b) {
            p.push_back(d->GetDipolePiece(b));
            s.push_back(d->GetDipoleStart(b));
            e.push_back(d->GetDipoleEnd(b));
        }
        check(gain_upload_dipole_pieces(engine_, (int)p.size(), p.data(), (int)d->GetMaxContracts(), s.data(),
                                        e.data()));
    }
    void TransferDipole(const double* piece, int N, int startF, int endF, int ncontrF) {
        check(gain_upload_dipole(engine_, piece, N, startF, endF, ncontrF));
        dipN_ = N;
        startF_ = startF;
        endF_ = endF;
        ncontrF_ = ncontrF;
        cudaFree(dipole_);
        dipole_ = upload(piece, (size_t)3 * N * ncontrF);
        doing_half_ls_ = true;
    }

    // BaseClasses/GpuManager.cpp:440-478: the Wigner tables of the last basis set, indexed by
    // dJ = J' - J'' + 1 (entries with rot == NULL are absent); WignerT has the reference
    // Wigner fields rot, nlevelsI, nlevelsF (common/Wigner.h)
    template <class WignerT>
    void TransferWigner(const std::vector<WignerT>& w) {
        if (!rotsym_) return;
        std::vector<Wigner> row(3);
        for (size_t dj = 0; dj < w.size() && dj < 3; ++dj) {
            if (!w[dj].rot) continue;
            Wigner& x = row[dj];
            x.nI = w[dj].nlevelsI;
            x.nF = w[dj].nlevelsF;
            const size_t n = (size_t)3 * x.nI * x.nF * maxdeg_ * maxdeg_;
            x.host.assign(w[dj].rot, w[dj].rot + n);
            x.rot = upload(w[dj].rot, n);
        }
        wigner_.push_back(row);
    }

    // BaseClasses/GpuManager.cpp:267-378
    void AllocateVectors(int nJ, int nsizemax, int dimenmax) {
        nsize_max_ = nsizemax;
        dimen_max_ = dimenmax;
        check_cuda(cudaMallocHost((void**)&host_vectorI_, sizeof(double) * nsizemax), "cudaMallocHost");
        vectorI_ = alloc(nsizemax);
        for (int j = 0; j < nJ; ++j) {
            prim_half_ls_.push_back({});
            half_ls_.push_back({});
            for (int d = 0; d < maxdeg_; ++d) {
                prim_half_ls_.back().push_back(alloc(dimenmax));
                half_ls_.back().push_back(alloc(dimenmax));
            }
        }
        for (int p = 0; p < nprocs_; ++p) {
            double* h;
            check_cuda(cudaMallocHost((void**)&h, sizeof(double) * nsizemax), "cudaMallocHost");
            host_vectorF_.push_back(h);
            check_cuda(cudaMallocHost((void**)&h, sizeof(double) * maxdeg_ * maxdeg_), "cudaMallocHost");
            host_ls_.push_back(h);
            vectorF_.push_back(alloc(nsizemax));
            prim_vectorF_.push_back(alloc(dimenmax));
            ls_.push_back(alloc((size_t)maxdeg_ * maxdeg_));
        }
    }

    double* GetInitialVector() { return host_vectorI_; }
    double* GetFinalVector(int proc) { return host_vectorF_.at(proc); }
    double* GetLinestrength(int proc) { return host_ls_.at(proc); }
    bool WillDoHalfLs() const { return doing_half_ls_; }
    int GetCurrentBlock() const { return current_block_; }

    // :537-545
    void UpdateEigenVector() {
        check_cuda(cudaMemcpy(vectorI_, host_vectorI_, sizeof(double) * nsize_max_, cudaMemcpyHostToDevice),
                   "UpdateEigenVector");
    }
    void UpdateEigenVector(int proc) {
        check_cuda(cudaMemcpyAsync(vectorF_[proc], host_vectorF_[proc], sizeof(double) * nsize_max_,
                                   cudaMemcpyHostToDevice, dot_stream_[proc]),
                   "UpdateEigenVector(proc)");
    }
    // :761-766
    void ResetHalfLinestrength(int indF, int idegI) {
        check_cuda(cudaMemset(half_ls_[indF][idegI], 0, sizeof(double) * dimen_max_), "ResetHalfLinestrength");
    }
    // :612-622 (+ TransformHalfLsVector :625-641, ExecuteKBlockHalfLs :645-732)
    void ExecuteHalfLs(int indI, int indF, int idegI, int igammaI) {
        Basis& bI = bases_.at(indI);
        Basis& bF = bases_.at(indF);
        Inflation& fI = infl_.at(indI);
        check(gain_expand(bI.dimen, igammaI, fI.maxcoeff, idegI, fI.sdeg[igammaI], fI.Ntot[igammaI], fI.ijterms,
                          fI.icontr, fI.N[igammaI], fI.repres[igammaI], vectorI_, prim_half_ls_[indF][idegI],
                          nullptr));
        if (rotsym_) {   // ExecuteRotSymHalfLs, :547-610
            const Wigner& w = wigner_at(indI, bF.J - bI.J + 1);
            check(gain_hls_rotsym(bF.dimen, bI.dimen, w.nI, w.nF, maxdeg_, bI.K, bF.K, bI.lev, bF.lev, bI.vib, bF.vib,
                                  startF_, endF_, ncontrF_, dipole_, w.rot, prim_half_ls_[indF][idegI],
                                  half_ls_[indF][idegI], dipN_, nullptr));
            check_cuda(cudaDeviceSynchronize(), "ExecuteHalfLs");
            return;
        }
        for (int kF = 0; kF < bF.J + 1; ++kF)
            check(gain_hls_kblock(bF.host_kblock[kF], bI.dimen, bI.J, bF.J, kF, bI.tau, bF.tau, bI.vib, bF.vib,
                                  bF.kstart[kF], bI.kstart[std::max(kF - 1, 0)], startF_, endF_, ncontrF_,
                                  bF.host_kblock[kF], bI.kblock, dipole_, prim_half_ls_[indF][idegI], threej_,
                                  half_ls_[indF][idegI], jmax_, dipN_, nullptr));
        check_cuda(cudaDeviceSynchronize(), "ExecuteHalfLs");
    }
    void GetHalfLineStrengthResult(double* half_ls, int indF, int idegI) {
        check_cuda(cudaMemcpy(half_ls, half_ls_[indF][idegI], sizeof(double) * bases_.at(indF).dimen,
                              cudaMemcpyDeviceToHost),
                   "GetHalfLineStrengthResult");
    }
    void UpdateHalfLinestrength(double* half_ls, int jInd, int ideg) {
        check_cuda(cudaMemcpy(half_ls_[jInd][ideg], half_ls, sizeof(double) * dimen_max_, cudaMemcpyHostToDevice),
                   "UpdateHalfLinestrength");
    }
    // :733-746
    void ExecuteDotProduct(int indF, int idegI, int idegF, int igammaF, int proc) {
        Basis& bF = bases_.at(indF);
        Inflation& fF = infl_.at(indF);
        check(gain_expand(bF.dimen, igammaF, fF.maxcoeff, idegF, fF.sdeg[igammaF], fF.Ntot[igammaF], fF.ijterms,
                          fF.icontr, fF.N[igammaF], fF.repres[igammaF], vectorF_[proc], prim_vectorF_[proc],
                          dot_stream_[proc]));
        check(gain_dot(bF.dimen, prim_vectorF_[proc], half_ls_[indF][idegI], ls_[proc] + idegI + idegF * maxdeg_,
                       dot_stream_[proc]));
    }
    // :755-759
    void WaitForLineStrengthResult(int proc) {
        check_cuda(cudaMemcpyAsync(host_ls_[proc], ls_[proc], sizeof(double) * maxdeg_ * maxdeg_,
                                   cudaMemcpyDeviceToHost, dot_stream_[proc]),
                   "WaitForLineStrengthResult");
        check_cuda(cudaStreamSynchronize(dot_stream_[proc]), "WaitForLineStrengthResult");
    }
    void WaitForDevice() { check_cuda(cudaDeviceSynchronize(), "WaitForDevice"); }

    // Batched replacement of the per-transition loop for one block pair: eigenvectors of
    // both blocks must have been given with UploadEigenvectors; amplitudes stay on the device
    // (gain_pair_amp_device) or come back with gain_fetch_amp(engine(), ...).
    void UploadEigenvectors(int jind, int gamma, int nlevels, int nsize, const double* vecs) {
        check(gain_upload_eigvecs(engine_, jind, gamma, nlevels, nsize, vecs));
    }
    gain_stats ExecuteBlockPair(const gain_pair_job& job, gain_path path, const gain_split_opts* opts = nullptr) {
        send_wigner(job);
        gain_stats st{};
        check(gain_run_pair(engine_, &job, path, opts, &st));
        return st;
    }
    // A block pair of degenerate symmetries: every component pair (idegI, idegF) that passes
    // the degeneracy filter, kept in the engine's component slots; gain_pair_lines with the
    // states' ndegI / ndegF then sums them as OutputLinestrength does.
    gain_stats ExecuteBlockPairDegenerate(const gain_pair_job& job, const gain_filters& filters, gain_path path,
                                          const gain_split_opts* opts = nullptr) {
        send_wigner(job);
        gain_stats st{};
        check(gain_run_pair_degenerate(engine_, &job, &filters, path, opts, &st));
        return st;
    }
    gain_engine engine() const { return engine_; }

   private:
    void send_wigner(const gain_pair_job& job) {
        if (!rotsym_) return;
        // the pair's rotational matrix elements, once per (J'', J') pair
        const int key = job.jindI * 100000 + job.jindF;
        if (std::find(wigner_sent_.begin(), wigner_sent_.end(), key) == wigner_sent_.end()) {
            const Wigner& w = wigner_at(job.jindI, bases_.at(job.jindF).J - bases_.at(job.jindI).J + 1);
            check(gain_upload_wigner(engine_, job.jindI, job.jindF, w.nI, w.nF, maxdeg_, w.host.data()));
            wigner_sent_.push_back(key);
        }
    }
    struct Basis {
        int J = 0, dimen = 0;
        int *tau = nullptr, *vib = nullptr, *kblock = nullptr, *K = nullptr, *lev = nullptr;
        std::vector<int> host_kblock, kstart;
    };
    struct Wigner {
        int nI = 0, nF = 0;
        double* rot = nullptr;
        std::vector<double> host;
    };
    const Wigner& wigner_at(int indI, int dj) const {
        if (indI < 0 || indI >= (int)wigner_.size() || dj < 0 || dj > 2 || !wigner_[indI][dj].rot)
            throw Error(GAIN_ERR_NOT_READY, "no Wigner table for this basis pair (TransferWigner)");
        return wigner_[indI][dj];
    }
    struct Inflation {
        int maxcoeff = 0;
        int *ijterms = nullptr, *icontr = nullptr;
        std::vector<int*> N;
        std::vector<double*> repres;
        std::vector<int> Ntot, sdeg;
    };

    template <class T>
    T* upload(const T* h, size_t n) {
        T* d = nullptr;
        check_cuda(cudaMalloc((void**)&d, sizeof(T) * std::max<size_t>(n, 1)), "cudaMalloc");
        owned_.push_back(d);
        if (n) check_cuda(cudaMemcpy(d, h, sizeof(T) * n, cudaMemcpyHostToDevice), "cudaMemcpy");
        return d;
    }
    double* alloc(size_t n) {
        double* d = nullptr;
        check_cuda(cudaMalloc((void**)&d, sizeof(double) * std::max<size_t>(n, 1)), "cudaMalloc");
        owned_.push_back(d);
        check_cuda(cudaMemset(d, 0, sizeof(double) * std::max<size_t>(n, 1)), "cudaMemset");
        return d;
    }
    void release() {
        for (void* p : owned_) cudaFree(p);
        owned_.clear();
        if (dipole_) cudaFree(dipole_);
        dipole_ = nullptr;
        if (host_vectorI_) cudaFreeHost(host_vectorI_);
        for (double* h : host_vectorF_) cudaFreeHost(h);
        for (double* h : host_ls_) cudaFreeHost(h);
        for (cudaStream_t s : dot_stream_) cudaStreamDestroy(s);
        host_vectorI_ = nullptr;
        host_vectorF_.clear();
        host_ls_.clear();
        dot_stream_.clear();
        if (engine_) gain_engine_destroy(engine_);
        engine_ = nullptr;
    }

    int gpu_id_, nprocs_;
    bool rotsym_ = false;
    std::vector<std::vector<Wigner>> wigner_;
    std::vector<int> wigner_sent_;
    int jmax_ = 0, nsym_ = 0, maxdeg_ = 1;
    gain_engine engine_ = nullptr;
    double* threej_ = nullptr;
    double* dipole_ = nullptr;
    int dipN_ = 0, startF_ = 0, endF_ = 0, ncontrF_ = 0;
    bool doing_half_ls_ = false;
    int current_block_ = 0;
    std::function<void(int, const double**, int*, int*, int*, int*)> switch_piece_;
    int nsize_max_ = 0, dimen_max_ = 0;
    std::vector<Basis> bases_;
    std::vector<Inflation> infl_;
    double* host_vectorI_ = nullptr;
    double* vectorI_ = nullptr;
    std::vector<std::vector<double*>> prim_half_ls_, half_ls_;
    std::vector<double*> host_vectorF_, host_ls_, vectorF_, prim_vectorF_, ls_;
    std::vector<cudaStream_t> dot_stream_;
    std::vector<void*> owned_;
};

}  // namespace gain
