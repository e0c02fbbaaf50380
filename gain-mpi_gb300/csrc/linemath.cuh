// S, A and I of one line (BaseClasses/Output.cpp:52-112), shared by the line
// assembly (k_lines) and the line-list text kernels so both see the same doubles.
#pragma once
#include "gain_internal.h"

namespace gain {

struct LineVals {
    double nu, ls, A, I;
    double e2;  // exp(-beta nu) as the intensity used it (0 without the intensity)
    int keep;   // the reference writes the line: nu in FREQ-WINDOW, nu >= 1e-40, A >= THRESH_LINE
};

// The line strength of the line at amp[off] (and its component slots).
__device__ __forceinline__ double line_ls(const double* amp, long off, const LineParams& p) {
    if (p.nslot == 0) {
        const double a = amp[off];
        return __dmul_rn(a, a);                               // :83, ndegI = ndegF = 1
    }
    double ls = 0.0;
    for (int s = 0; s < p.nslot; ++s) {                       // :78-85
        const double a = amp[off + (long)p.slot[s] * p.slot_stride];
        ls = __dadd_rn(ls, __dmul_rn(a, a));
    }
    ls = __ddiv_rn(ls, (double)p.ndegI);                      // :89
    if (p.reduced_deg) ls = __dmul_rn(ls, (double)p.ndegI);   // :90-91
    return ls;
}

__device__ __forceinline__ LineVals line_eval(const double* amp, long off, double eIr, double eFc,
                                              const LineParams& p) {
    LineVals v;
    v.nu = eFc - eIr;
    v.ls = line_ls(amp, off, p);
    const double anu = fabs(v.nu);
    v.A = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(p.acoef_2jI1, v.ls), anu), anu), anu);   // :93
    v.keep = (v.nu >= p.freq_lo && v.nu <= p.freq_hi && v.nu >= 1e-40 && v.A >= p.thresh) ? 1 : 0;
    v.I = 0.0;
    v.e2 = 0.0;
    if (p.with_intensity && v.nu >= 1e-40) {
        // CMCOEF*A*gns*(2jF+1)*exp(-beta E'')*(1-exp(-beta nu))/(nu^2 Q), :101-102
        double t = __dmul_rn(p.cmcoef, v.A);
        t = __dmul_rn(t, p.gnsF);
        t = __dmul_rn(t, p.two_jF1);
        t = __dmul_rn(t, exp(-p.beta * (eIr - p.zpe)));
        v.e2 = exp(-p.beta * v.nu);
        t = __dmul_rn(t, 1.0 - v.e2);
        v.I = __ddiv_rn(t, __dmul_rn(__dmul_rn(v.nu, v.nu), p.q_part));
    }
    return v;
}

}  // namespace gain
