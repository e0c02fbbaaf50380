// Drives gain::GpuManager (include/gain_gpu_manager.hpp) the way GAIN-MPI's main.cpp drives
// its GpuManager (main.cpp:172-336), on one block pair read from a flat binary file, and
// writes the amplitude of every (lower, upper) pair.  Built and run by tests/test_gpu_manager.py.
//
// input (little-endian int32 / float64 records, written by the test):
//   ints:  nv jmax nsym JI JF gI gF nlower nupper startF endF
//   per J (I then F): dimen, K[dimen], ktau[dimen], vib[dimen], kblock[J+1], kstart[J+1],
//                     icontr[2 dimen], ijterms[dimen nsym], N[nsym][dimen], Ntot[nsym]
//   doubles: dipole piece [3 nv (endF-startF)], lower vectors [nlower NtotI],
//            upper vectors [nupper NtotF]
//   optional: int rotsym (1), ints nlevelsI nlevelsF, doubles rot[3 nlevelsI nlevelsF] -- the
//             rotational-symmetry form, with the Wigner table of the pair JI -> JF
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "gain_gpu_manager.hpp"

namespace {
FILE* fin;
int geti() { int v; if (fread(&v, 4, 1, fin) != 1) { fprintf(stderr, "short read\n"); exit(2); } return v; }
std::vector<int> getiv(size_t n) { std::vector<int> v(n); if (n && fread(v.data(), 4, n, fin) != n) exit(2); return v; }
std::vector<double> getdv(size_t n) { std::vector<double> v(n); if (n && fread(v.data(), 8, n, fin) != n) exit(2); return v; }
struct Wig { double* rot; int nlevelsI, nlevelsF; };   // the fields of the reference's Wigner
// The reference Dipole's getters over a dipole split into nblocks pieces of the upper index
// (TroveDipole.cpp:85-112: ceil(ncontr / nblocks) functions per piece, flipped layout).
struct BlockedDipole {
    int n;
    std::vector<int> s, e;
    std::vector<std::vector<double>> pieces;
    BlockedDipole(const std::vector<double>& full, int nv, int nblocks) : n(nv) {
        const int per = (int)ceilf((float)nv / (float)nblocks);
        for (int b = 0; b < nblocks; ++b) {
            const int s0 = b * per, e0 = std::min((b + 1) * per, nv), c = e0 - s0;
            s.push_back(s0);
            e.push_back(e0);
            std::vector<double> p((size_t)3 * nv * c);
            for (int k = 0; k < 3; ++k)
                for (int i = 0; i < nv; ++i)
                    for (int f = s0; f < e0; ++f)
                        p[(f - s0) + (size_t)i * c + (size_t)k * nv * c] = full[f + (size_t)i * nv + (size_t)k * nv * nv];
            pieces.push_back(std::move(p));
        }
    }
    const double* GetDipolePiece(int b) { return pieces[b].data(); }
    size_t GetMaxContracts() { return (size_t)n; }
    int GetDipoleStart(int b) { return s[b]; }
    int GetDipoleEnd(int b) { return e[b]; }
    int GetDipoleNcontr(int b) { return e[b] - s[b]; }
    int GetNumBlocks() { return (int)pieces.size(); }
};
struct J { int J, dimen; std::vector<int> K, ktau, vib, kblock, kstart, icontr, ijterms, Ntot; std::vector<std::vector<int>> N; };
}

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s input output [dipole_blocks]\n", argv[0]); return 1; }
    const int nblocks = argc > 3 ? atoi(argv[3]) : 1;
    fin = fopen(argv[1], "rb");
    if (!fin) return 1;
    const int nv = geti(), jmax = geti(), nsym = geti(), JI = geti(), JF = geti(), gI = geti(), gF = geti();
    const int nlower = geti(), nupper = geti(), startF = geti(), endF = geti();
    J js[2];
    for (int t = 0; t < 2; ++t) {
        J& j = js[t];
        j.J = t == 0 ? JI : JF;
        j.dimen = geti();
        j.K = getiv(j.dimen); j.ktau = getiv(j.dimen); j.vib = getiv(j.dimen);
        j.kblock = getiv(j.J + 1); j.kstart = getiv(j.J + 1);
        j.icontr = getiv(2 * (size_t)j.dimen); j.ijterms = getiv((size_t)j.dimen * nsym);
        for (int g = 0; g < nsym; ++g) j.N.push_back(getiv(j.dimen));
        j.Ntot = getiv(nsym);
    }
    std::vector<double> piece = getdv((size_t)3 * nv * (endF - startF));
    std::vector<double> vl = getdv((size_t)nlower * js[0].Ntot[gI]);
    std::vector<double> vu = getdv((size_t)nupper * js[1].Ntot[gF]);
    int rotsym = 0, nlevI = 0, nlevF = 0;
    std::vector<double> rot;
    if (fread(&rotsym, 4, 1, fin) == 1 && rotsym) {
        nlevI = geti();
        nlevF = geti();
        rot = getdv((size_t)3 * nlevI * nlevF);
    }
    fclose(fin);
    try {
        gain::GpuManager gpu(0, 1, rotsym != 0);
        gpu.InitializeAndTransferConstants(jmax, nsym, 1);
        std::unique_ptr<BlockedDipole> blocked;
        if (nblocks > 1) {   // MultiGpuManager::TransferDipole: the device starts with block 0
            if (startF != 0 || endF != nv) { fprintf(stderr, "blocks need the whole dipole\n"); return 1; }
            blocked.reset(new BlockedDipole(piece, nv, nblocks));
            gpu.TransferDipole(blocked.get(), 0);
        } else {
            gpu.TransferDipole(piece.data(), nv, startF, endF, endF - startF);
        }
        int dimen_max = 0, nsize_max = 0;
        for (int t = 0; t < 2; ++t) {
            J& j = js[t];
            gpu.TransferBasisSet(j.J, j.dimen, j.K.data(), j.ktau.data(), j.vib.data(), j.kblock.data(), j.kstart.data());
            if (rotsym) {   // main.cpp:193, after each basis set: its tables by dJ = J' - J + 1
                std::vector<Wig> w(3, Wig{nullptr, 0, 0});
                if (t == 0) w[JF - JI + 1] = Wig{rot.data(), nlevI, nlevF};
                gpu.TransferWigner(w);
            }
            std::vector<double*> repres;
            std::vector<std::vector<double>> ones;
            std::vector<int*> N;
            for (int g = 0; g < nsym; ++g) {
                ones.emplace_back(std::max(1, j.Ntot[g]), 1.0);
                N.push_back(j.N[g].data());
                nsize_max = std::max(nsize_max, j.Ntot[g]);
            }
            for (auto& o : ones) repres.push_back(o.data());
            gpu.TransferInflation(j.icontr.data(), j.ijterms.data(), j.dimen, j.dimen, 1, repres, N, j.Ntot,
                                  std::vector<int>(nsym, 1));
            dimen_max = std::max(dimen_max, j.dimen);
        }
        gpu.AllocateVectors(2, nsize_max, dimen_max);
        std::vector<double> amp((size_t)nlower * nupper);
        for (int l = 0; l < nlower; ++l) {                  // main.cpp:238 lower-state loop
            std::copy(vl.begin() + (size_t)l * js[0].Ntot[gI], vl.begin() + (size_t)(l + 1) * js[0].Ntot[gI],
                      gpu.GetInitialVector());
            gpu.UpdateEigenVector();
            gpu.ResetHalfLinestrength(1, 0);
            for (int b = 0; b < nblocks; ++b) {             // MultiGpuManager::ExecuteHalfLs block loop
                if (nblocks > 1 && gpu.GetCurrentBlock() != b) gpu.SwitchDipoleBlock(b);
                gpu.ExecuteHalfLs(0, 1, 0, gI);
            }
            for (int u = 0; u < nupper; ++u) {              // main.cpp:293 upper-state loop
                std::copy(vu.begin() + (size_t)u * js[1].Ntot[gF], vu.begin() + (size_t)(u + 1) * js[1].Ntot[gF],
                          gpu.GetFinalVector(0));
                gpu.UpdateEigenVector(0);
                gpu.ExecuteDotProduct(1, 0, 0, gF, 0);
                gpu.WaitForLineStrengthResult(0);
                amp[(size_t)l * nupper + u] = gpu.GetLinestrength(0)[0];
            }
        }
        FILE* fo = fopen(argv[2], "wb");
        fwrite(amp.data(), 8, amp.size(), fo);
        fclose(fo);
    } catch (const gain::Error& e) {
        fprintf(stderr, "gain error: %s\n", e.what());
        return 3;
    }
    return 0;
}
