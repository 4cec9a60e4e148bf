// J2 (von Mises, linear isotropic/kinematic hardening) return mapping and its
// consistent tangent, shared by the explicit, Newmark and ExtendedNewmark
// device paths.  Device code only; include from .cu files.
#pragma once
#include <cuda_runtime.h>

namespace svl {

constexpr int kJ2State = 13;   // plastic strain (6), back stress (6), alpha

// J2 radial return on the tensor strain E[6] (shear = gamma/2), in place on
// the Gauss-point state (PlasticPlaneStrainJ2.cpp:227-279, Plastic3DJ2.cpp:206-255).
// Consistent tangent of the return mapping (PlasticPlaneStrainJ2.cpp:276,
// Plastic3DJ2.cpp): K 1(x)1 + 2G Id for an elastic step, else
// K 1(x)1 + 2G (Id - c1 n(x)n) - c2 (Id - n(x)n), c1 = 1/(1 + H/(3G)),
// c2 = 4 G^2 dg / |xi|; Id = I - 1(x)1/3 with I = diag(1,1,1,1/2,1/2,1/2).
// Stored entry by entry in [entry][ngp][E] order: 2D keeps rows/cols 1,2,4.
template <int ND>
__device__ __forceinline__ void j2_store_tangent(double* ct, size_t stride, double K, double G, bool plastic,
                                                 const double n[6], double c1, double c2) {
    constexpr int NS = ND == 2 ? 3 : 6;
    const int ix[6] = {ND == 2 ? 1 : 0, ND == 2 ? 2 : 1, ND == 2 ? 4 : 2, 3, 4, 5};
#pragma unroll
    for (int a = 0; a < NS; ++a)
#pragma unroll
        for (int b = 0; b < NS; ++b) {
            const int i = ix[a], j = ix[b];
            const double D = (i < 3 && j < 3) ? 1.0 : 0.0;
            const double I = (i == j) ? (i < 3 ? 1.0 : 0.5) : 0.0;
            const double Id = I - 1.0 / 3.0 * D;
            double v;
            if (!plastic) v = K * D + 2.0 * G * Id;
            else {
                const double nn = n[i] * n[j];
                v = K * D + 2.0 * G * (Id - c1 * nn) - c2 * (Id - nn);
            }
            ct[(size_t)(a * NS + b) * stride] = v;
        }
}

template <int ND = 3>
__device__ __forceinline__ void j2_return(const double E[6], double st[kJ2State], double K, double G,
                                          double H, double beta, double SY, double sig6[6],
                                          double* ct = nullptr, size_t ct_stride = 0) {
    const double tr = E[0] + E[1] + E[2];
    double trial[6], rel[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const double dev = E[i] - (i < 3 ? 1.0 / 3.0 * tr : 0.0);
        trial[i] = 2.0 * G * (dev - st[i]);
        rel[i] = trial[i] - st[6 + i];
    }
    const double nrm = sqrt(rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2] +
                            2.0 * (rel[3] * rel[3] + rel[4] * rel[4] + rel[5] * rel[5]));
    const double f = nrm - sqrt(2.0 / 3.0) * (SY + st[12] * beta * H);
    if (f <= 0) {
#pragma unroll
        for (int i = 0; i < 6; ++i) sig6[i] = (i < 3 ? K * tr : 0.0) + trial[i];
        if (ct) {
            const double z[6] = {0, 0, 0, 0, 0, 0};
            j2_store_tangent<ND>(ct, ct_stride, K, G, false, z, 0.0, 0.0);
        }
    } else {
        const double dg = f / (2.0 * G + 2.0 / 3.0 * H);
        st[12] += sqrt(2.0 / 3.0) * dg;
        double nv[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const double n = rel[i] / nrm;
            nv[i] = n;
            st[6 + i] += 2.0 / 3.0 * (1.0 - beta) * H * dg * n;
            st[i] += dg * n;
            sig6[i] = (i < 3 ? K * tr : 0.0) + trial[i] - 2.0 * G * dg * n;
        }
        if (ct) j2_store_tangent<ND>(ct, ct_stride, K, G, true, nv, 1.0 / (1.0 + H / G / 3.0), 4.0 * G * G * dg / nrm);
    }
}

}  // namespace svl
