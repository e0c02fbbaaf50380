// ORACLE (test infrastructure only): runs the reference's own, unmodified GPU kernels.
//
// The reference's GPU/dipole_GPU.cu is compiled, unchanged, into oracle/_ref/dipole_GPU.cubin
// by oracle/build_ref.sh.  This harness loads that cubin through the CUDA driver API and
// drives it exactly the way BaseClasses/GpuManager.cpp does for one block pair:
//   * constants: dip_stride_1 = Dipole::GetMaxContracts (:514), c_jmax (:189);
//   * per lower state: reset half_ls (:761-766), device_expand_vectors on the lower vector
//     (TransformHalfLsVector, :625-641; grid ceil(dimen/512) x 512, dipole_GPU.cu:139),
//     one device_compute_1st_half_ls_flipped_dipole_shared_block_nontrove launch per kF
//     (ExecuteKBlockHalfLs, :651-709; grid ceil(kblock/128) x 128, dipole_GPU.cu:191);
//   * per upper state: device_expand_vectors on the upper vector, then cublasDdot with the
//     device pointer mode (ExecuteDotProduct, :733-746), then the D2H of the result and a
//     stream synchronisation (WaitForLineStrengthResult, :755-759).
// It produces golden half_ls vectors and amplitudes, and times the reference's per-transition
// loop.  Only the tests and fixture scripts use it.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cublas_v2.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

const char* kHlsName =
    "_Z63device_compute_1st_half_ls_flipped_dipole_shared_block_nontroveiiiiiPKiS0_S0_S0_iiiiiS0_PKdS2_S2_Pd";
const char* kExpandName = "_Z21device_expand_vectorsiiiiiiPKiS0_S0_PKdS2_Pd";
const char* kRotsymName =
    "_Z64device_compute_1st_half_ls_flipped_dipole_shared_rotsym_nontroveiiiiiPKiS0_S0_S0_S0_S0_iiiPKdS2_S2_Pd";

CUmodule g_mod = nullptr;
CUfunction g_hls = nullptr, g_expand = nullptr, g_rotsym = nullptr;
CUdeviceptr g_dip_stride = 0, g_jmax = 0;
char g_err[512];

#define RT(x)                                                                         \
    do {                                                                              \
        cudaError_t e_ = (x);                                                         \
        if (e_ != cudaSuccess) {                                                      \
            snprintf(g_err, sizeof g_err, "%s: %s", #x, cudaGetErrorString(e_));      \
            return -1;                                                                \
        }                                                                             \
    } while (0)
#define DRV(x)                                                                        \
    do {                                                                              \
        CUresult e_ = (x);                                                            \
        if (e_ != CUDA_SUCCESS) {                                                     \
            const char* s_ = nullptr;                                                 \
            cuGetErrorString(e_, &s_);                                                \
            snprintf(g_err, sizeof g_err, "%s: %s", #x, s_ ? s_ : "?");               \
            return -1;                                                                \
        }                                                                             \
    } while (0)

template <class T>
int upload(T** d, const T* h, size_t n) {
    RT(cudaMalloc((void**)d, sizeof(T) * (n ? n : 1)));
    if (n) RT(cudaMemcpy(*d, h, sizeof(T) * n, cudaMemcpyHostToDevice));
    return 0;
}

}  // namespace

extern "C" {

struct refh_pair {
    int jI, jF, jmax;
    int dimenI, dimenF;
    const int *tauI, *tauF, *icorrI, *icorrF;
    const int *kstartI, *kblockI, *kstartF, *kblockF;
    int gammaI, gammaF;
    int maxcoeffI, maxcoeffF, NtotI, NtotF, nsymI, nsymF, matsizeI, matsizeF;
    const int *ijtermsI, *icontrI, *NI;
    const double* represI;
    const int *ijtermsF, *icontrF, *NF;
    const double* represF;
    const double* dipole_me;
    int dip_stride, startFblock, endFblock, ncontrF;
    const double* threej;
    int nlower, nupper;
    const double* vec_lower;
    const double* vec_upper;
    int idegI, idegF, sdegI, sdegF;   // degenerate components and degeneracies (0 reads as 1)
};

const char* refh_error(void) { return g_err; }

int refh_init(const char* cubin_path) {
    if (g_mod) return 0;
    RT(cudaFree(0));  // creates and binds the primary context the driver calls below use
    DRV(cuModuleLoad(&g_mod, cubin_path));
    DRV(cuModuleGetFunction(&g_hls, g_mod, kHlsName));
    DRV(cuModuleGetFunction(&g_expand, g_mod, kExpandName));
    DRV(cuModuleGetFunction(&g_rotsym, g_mod, kRotsymName));
    size_t sz = 0;
    DRV(cuModuleGetGlobal(&g_dip_stride, &sz, g_mod, "dip_stride_1"));
    DRV(cuModuleGetGlobal(&g_jmax, &sz, g_mod, "c_jmax"));
    return 0;
}

// amp: [nlower][nupper]; hls: optional [nlower][dimenF]; seconds: optional wall time of the
// upper-state loop (the reference's per-transition path), summed over lower states.
int refh_run_pair(const refh_pair* p, double* amp, double* hls, double* seconds) {
    if (!g_mod) {
        snprintf(g_err, sizeof g_err, "refh_init not called");
        return -1;
    }
    int jmax = p->jmax, stride = p->dip_stride;
    DRV(cuMemcpyHtoD(g_jmax, &jmax, sizeof(int)));
    DRV(cuMemcpyHtoD(g_dip_stride, &stride, sizeof(int)));

    int *d_tauI, *d_tauF, *d_icI, *d_icF, *d_kbI;
    int *d_ijI, *d_ctI, *d_NI, *d_ijF, *d_ctF, *d_NF;
    double *d_rpI, *d_rpF, *d_dip, *d_3j, *d_vecI, *d_vecF, *d_primI, *d_primF, *d_hls, *d_res;
    const size_t dipn = (size_t)3 * p->ncontrF * p->dip_stride;
    const int nj = (p->jmax + 1) * (p->jmax + 1) * 9;
    if (upload(&d_tauI, p->tauI, p->dimenI) || upload(&d_tauF, p->tauF, p->dimenF) ||
        upload(&d_icI, p->icorrI, p->dimenI) || upload(&d_icF, p->icorrF, p->dimenF) ||
        upload(&d_kbI, p->kblockI, p->jI + 1) ||
        upload(&d_ijI, p->ijtermsI, (size_t)p->maxcoeffI * p->nsymI) ||
        upload(&d_ctI, p->icontrI, (size_t)2 * p->dimenI) || upload(&d_NI, p->NI, p->maxcoeffI) ||
        upload(&d_rpI, p->represI, (size_t)p->NtotI * (p->sdegI > 0 ? p->sdegI : 1) * p->matsizeI) ||
        upload(&d_ijF, p->ijtermsF, (size_t)p->maxcoeffF * p->nsymF) ||
        upload(&d_ctF, p->icontrF, (size_t)2 * p->dimenF) || upload(&d_NF, p->NF, p->maxcoeffF) ||
        upload(&d_rpF, p->represF, (size_t)p->NtotF * (p->sdegF > 0 ? p->sdegF : 1) * p->matsizeF) ||
        upload(&d_dip, p->dipole_me, dipn) ||
        upload(&d_3j, p->threej, nj))
        return -1;
    RT(cudaMalloc(&d_vecI, sizeof(double) * p->NtotI));
    RT(cudaMalloc(&d_vecF, sizeof(double) * p->NtotF));
    RT(cudaMalloc(&d_primI, sizeof(double) * p->dimenI));
    RT(cudaMalloc(&d_primF, sizeof(double) * p->dimenF));
    RT(cudaMalloc(&d_hls, sizeof(double) * p->dimenF));
    RT(cudaMalloc(&d_res, sizeof(double)));
    double* h_vecF = nullptr;
    double* h_res = nullptr;
    RT(cudaMallocHost(&h_vecF, sizeof(double) * p->NtotF));
    RT(cudaMallocHost(&h_res, sizeof(double)));

    cudaStream_t st;
    RT(cudaStreamCreate(&st));
    cublasHandle_t h;
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
        snprintf(g_err, sizeof g_err, "cublasCreate failed");
        return -1;
    }
    cublasSetPointerMode(h, CUBLAS_POINTER_MODE_DEVICE);
    cublasSetStream(h, st);
    double total = 0.0;

    for (int l = 0; l < p->nlower; l++) {
        RT(cudaMemcpy(d_vecI, p->vec_lower + (size_t)l * p->NtotI, sizeof(double) * p->NtotI,
                      cudaMemcpyHostToDevice));
        RT(cudaMemset(d_hls, 0, sizeof(double) * p->dimenF));
        {
            int dimen = p->dimenI, g = p->gammaI, mc = p->maxcoeffI, ideg = p->idegI,
                sdeg = p->sdegI > 0 ? p->sdegI : 1, nt = p->NtotI;
            void* args[] = {&dimen, &g, &mc, &ideg, &sdeg, &nt, &d_ijI, &d_ctI, &d_NI, &d_rpI, &d_vecI, &d_primI};
            DRV(cuLaunchKernel(g_expand, (dimen + 511) / 512, 1, 1, 512, 1, 1, 0, st, args, nullptr));
        }
        for (int kF = 0; kF < p->jF + 1; kF++) {
            int dimenF = p->kblockF[kF], dimenI = p->dimenI, jI = p->jI, jF = p->jF, k = kF;
            int startF = p->kstartF[kF], startI = p->kstartI[kF - 1 > 0 ? kF - 1 : 0];
            int sFb = p->startFblock, eFb = p->endFblock, nc = p->ncontrF;
            void* args[] = {&dimenF, &dimenI, &jI, &jF, &k, &d_tauI, &d_tauF, &d_icI, &d_icF,
                            &startF, &startI, &sFb, &eFb, &nc, &d_kbI, &d_dip, &d_primI, &d_3j, &d_hls};
            if (dimenF > 0)
                DRV(cuLaunchKernel(g_hls, (dimenF + 127) / 128, 1, 1, 128, 1, 1, 0, st, args, nullptr));
        }
        RT(cudaStreamSynchronize(st));
        if (hls)
            RT(cudaMemcpy(hls + (size_t)l * p->dimenF, d_hls, sizeof(double) * p->dimenF,
                          cudaMemcpyDeviceToHost));
        auto t0 = std::chrono::steady_clock::now();
        for (int u = 0; u < p->nupper; u++) {
            memcpy(h_vecF, p->vec_upper + (size_t)u * p->NtotF, sizeof(double) * p->NtotF);
            RT(cudaMemcpyAsync(d_vecF, h_vecF, sizeof(double) * p->NtotF, cudaMemcpyHostToDevice, st));
            int dimen = p->dimenF, g = p->gammaF, mc = p->maxcoeffF, ideg = p->idegF,
                sdeg = p->sdegF > 0 ? p->sdegF : 1, nt = p->NtotF;
            void* args[] = {&dimen, &g, &mc, &ideg, &sdeg, &nt, &d_ijF, &d_ctF, &d_NF, &d_rpF, &d_vecF, &d_primF};
            DRV(cuLaunchKernel(g_expand, (dimen + 511) / 512, 1, 1, 512, 1, 1, 0, st, args, nullptr));
            if (cublasDdot(h, p->dimenF, d_primF, 1, d_hls, 1, d_res) != CUBLAS_STATUS_SUCCESS) {
                snprintf(g_err, sizeof g_err, "cublasDdot failed");
                return -1;
            }
            RT(cudaMemcpyAsync(h_res, d_res, sizeof(double), cudaMemcpyDeviceToHost, st));
            RT(cudaStreamSynchronize(st));
            amp[(size_t)l * p->nupper + u] = *h_res;
        }
        total += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (seconds) *seconds = total;
    cublasDestroy(h);
    cudaStreamDestroy(st);
    cudaFreeHost(h_vecF);
    cudaFreeHost(h_res);
    void* ptrs[] = {d_tauI, d_tauF, d_icI, d_icF, d_kbI, d_ijI, d_ctI, d_NI, d_ijF, d_ctF, d_NF,
                    d_rpI, d_rpF, d_dip, d_3j, d_vecI, d_vecF, d_primI, d_primF, d_hls, d_res};
    for (void* q : ptrs) cudaFree(q);
    RT(cudaGetLastError());
    return 0;
}

// The rotational-symmetry half line strength of one primitive lower vector, as
// GpuManager::ExecuteRotSymHalfLs launches it (BaseClasses/GpuManager.cpp:564-592) through
// compute_gpu_half_linestrength_rotsym_ (GPU/dipole_GPU.cu:238-262: grid ceil(dimenF/128) x
// 128), after the reset to zero of the half line strength (:761-766).  dipole: 3 x
// dip_stride x ncontrF doubles; wigner: 3 nlevelI nlevelF maxdeg^2 doubles.
int refh_hls_rotsym(int dimenF, int dimenI, int nlevelI, int nlevelF, int maxdeg, const int* kI, const int* kF,
                    const int* ktauI, const int* ktauF, const int* icorrI, const int* icorrF, int startFblock,
                    int endFblock, int ncontrF, const double* dipole, int dip_stride, const double* wigner,
                    const double* vector, double* half_ls) {
    if (!g_mod) {
        snprintf(g_err, sizeof g_err, "refh_init not called");
        return -1;
    }
    int stride = dip_stride;
    DRV(cuMemcpyHtoD(g_dip_stride, &stride, sizeof(int)));
    int *d_kI, *d_kF, *d_tI, *d_tF, *d_cI, *d_cF;
    double *d_dip, *d_w, *d_v, *d_h;
    const size_t wn = (size_t)3 * nlevelI * nlevelF * maxdeg * maxdeg;
    if (upload(&d_kI, kI, dimenI) || upload(&d_kF, kF, dimenF) || upload(&d_tI, ktauI, dimenI) ||
        upload(&d_tF, ktauF, dimenF) || upload(&d_cI, icorrI, dimenI) || upload(&d_cF, icorrF, dimenF) ||
        upload(&d_dip, dipole, (size_t)3 * dip_stride * ncontrF) || upload(&d_w, wigner, wn) ||
        upload(&d_v, vector, dimenI))
        return -1;
    RT(cudaMalloc(&d_h, sizeof(double) * dimenF));
    RT(cudaMemset(d_h, 0, sizeof(double) * dimenF));
    int a0 = dimenF, a1 = dimenI, a2 = nlevelI, a3 = nlevelF, a4 = maxdeg, a5 = startFblock, a6 = endFblock,
        a7 = ncontrF;
    void* args[] = {&a0, &a1, &a2, &a3, &a4, &d_kI, &d_kF, &d_tI, &d_tF, &d_cI, &d_cF,
                    &a5, &a6, &a7, &d_dip, &d_w, &d_v, &d_h};
    DRV(cuLaunchKernel(g_rotsym, (dimenF + 127) / 128, 1, 1, 128, 1, 1, 0, nullptr, args, nullptr));
    RT(cudaDeviceSynchronize());
    RT(cudaMemcpy(half_ls, d_h, sizeof(double) * dimenF, cudaMemcpyDeviceToHost));
    void* ptrs[] = {d_kI, d_kF, d_tI, d_tF, d_cI, d_cF, d_dip, d_w, d_v, d_h};
    for (void* q : ptrs) cudaFree(q);
    RT(cudaGetLastError());
    return 0;
}

}  // extern "C"
