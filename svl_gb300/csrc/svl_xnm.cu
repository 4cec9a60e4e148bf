// ExtendedNewmarkBeta with PML elements on the GPU (svl_xnm_*), and
// NewmarkBeta on the same elements (integrator SVL_XNM_NEWMARK: the increment
// terms in the effective force, no history matrix, the support-motion
// increment of step k - 1; NewmarkBeta.cpp:117-235).
//
// The reference assembles M, C, K and G once (ExtendedNewmarkBeta.cpp:64-70),
// re-assembles K and forms K + 4/dt^2 M + 2/dt C + dt/3 G every step
// (:233-245) and factorises it.  Here nothing is assembled: every operator
// application runs the element kernels on the vector and gathers the element
// vectors per total dof in element-tag order (an inverse connectivity, no
// atomics), so each total-dof sum has the reference's summation order.
//   solid elements (lin2DQuad4 / lin3DHexa8, elastic or J2, lumped mass):
//     y_e = K_e xK + ak_e K0_e (cK2 xK2) + diag(m_e) (sM xM + cM2 am_e xM2)
//     with K_e the tangent (stored at each J2 return mapping) and
//     C_e = am_e M_e + ak_e K0_e (Rayleigh with the initial stiffness);
//   PML elements: svl::pml_action_launch (svl_pml.cu) in gather mode.
// The solid element states and internal forces are updated by k_xstate from
// U + T dU after every solve (Algorithm::UpdateStatesIncrements); the next
// effective force reads the stored forces.  NewtonRaphson iterations repeat
// force, tangent solve and state update with the accumulated dU.
// With PML the effective matrix is symmetric indefinite (negative stress
// blocks of M), so the solve is MINRES (Paige & Saunders 1975) with the SPD
// preconditioner |diag(Keff)|^-1, restarted from its iterate until the true
// residual meets the tolerance.  Reductions are two-stage with a fixed block
// count, so results do not depend on scheduling.
// Operator applications (all element inputs one vector) use one thread per
// (element, Gauss point): k_xsolid_gp / k_pml_action_gp.  In the MINRES inner
// iterations they run in single precision on float tables and float element
// vectors (k_xgather_f); the restarts' true residual uses the double operator.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "svl_internal.hpp"
#include "svl_j2.cuh"

using namespace svl;

namespace {

#define XTRY(x) do { int st_ = (x); if (st_ != SVL_OK) return st_; } while (0)
#define XCUDA(x)                                                                         \
    do {                                                                                 \
        cudaError_t err_ = (x);                                                          \
        if (err_ != cudaSuccess) {                                                       \
            set_error("%s failed: %s (%s:%d)", #x, cudaGetErrorString(err_), __FILE__, __LINE__); \
            return SVL_ERR_CUDA;                                                         \
        }                                                                                \
    } while (0)

constexpr int kBlocks = 304, kThreads = 256;     // fixed two-stage reduction shape

struct XSolid {
    int n, ngp;
    const int32_t* edof;     // [n][NC]
    const int32_t* egeo;     // [n] geometry class
    const double* geo;       // [ngeo][ngp][NEN*ND + 1]  dN/dx and w t |J|
    const double* coef;      // [n][3] c1 c2 c3 of the initial elastic tangent
    const int32_t* kind;     // [n] 1 for a J2 element, or null (all elastic)
    const double* ctan;      // [NS*NS][ngp][n] J2 tangents of the last update
    const float* geo_f;      // single-precision copies for the single-precision
    const float* ctan_f;     // operator (conversions from double run at the FP64 rate)
    const float* opf;        // [n][NEN + 4] operator constants of Keff: m_a (4/dt^2 + 2/dt am),
                             // 2/dt ak, c1, c2, c3 (single-precision operator only)
    const float* xK_f;       // single-precision operator: the input vector and the
    float* y_f;              // element vectors in float (no filter, scale or accumulate)
    const double* ray;       // [n][2] am ak, or null
    const double* mlump;     // [n][NEN] row-sum lumped mass per element node
    const double *xK, *xK2, *xM, *xM2;   // total-dof inputs (null = 0)
    double cK2, sM, cM2, ftol, yscale;
    int accumulate;
    double* y;               // [n][NC]
};

// Strain (engineering shear) of the element vector u at one Gauss point.
template <int ND, int NEN, typename T>
__device__ __forceinline__ void xstrain(const T (&b)[NEN][3], const T* u, T ev[6]) {
#pragma unroll
    for (int i = 0; i < 6; ++i) ev[i] = 0.0;
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
        if (ND == 2) {
            ev[0] += b[a][0] * u[2 * a];
            ev[1] += b[a][1] * u[2 * a + 1];
            ev[2] += b[a][1] * u[2 * a] + b[a][0] * u[2 * a + 1];
        } else {
            const T ux = u[3 * a], uy = u[3 * a + 1], uz = u[3 * a + 2];
            ev[0] += b[a][0] * ux;
            ev[1] += b[a][1] * uy;
            ev[2] += b[a][2] * uz;
            ev[3] += b[a][1] * ux + b[a][0] * uy;
            ev[4] += b[a][2] * uy + b[a][1] * uz;
            ev[5] += b[a][2] * ux + b[a][0] * uz;
        }
    }
}
// y += w B^T sig (sig in the strain's order: 2D xx yy xy, 3D xx yy zz xy yz zx)
template <int ND, int NEN, typename T>
__device__ __forceinline__ void xbts(const T (&b)[NEN][3], T w, const T sig[6], T* y) {
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
        if (ND == 2) {
            y[2 * a] += w * (b[a][0] * sig[0] + b[a][1] * sig[2]);
            y[2 * a + 1] += w * (b[a][1] * sig[1] + b[a][0] * sig[2]);
        } else {
            const T bx = b[a][0], by = b[a][1], bz = b[a][2];
            y[3 * a] += w * (bx * sig[0] + by * sig[3] + bz * sig[5]);
            y[3 * a + 1] += w * (by * sig[1] + bx * sig[3] + bz * sig[4]);
            y[3 * a + 2] += w * (bz * sig[2] + by * sig[4] + bx * sig[5]);
        }
    }
}
// sig = C0 ev with the elastic coefficients c1 c2 c3
template <int ND, typename T>
__device__ __forceinline__ void xelastic(T c1, T c2, T c3, const T ev[6], T sig[6]) {
    if (ND == 2) {
        sig[0] = c1 * ev[0] + c2 * ev[1];
        sig[1] = c2 * ev[0] + c1 * ev[1];
        sig[2] = c3 * ev[2];
        sig[3] = sig[4] = sig[5] = 0.0;
    } else {
        sig[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
        sig[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
        sig[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
        sig[3] = c3 * ev[3]; sig[4] = c3 * ev[4]; sig[5] = c3 * ev[5];
    }
}

// Operator action of one J2 element: the stored tangent on xK, the initial
// elastic tangent on the stiffness-proportional damping input, lumped mass.
template <int ND, int NEN, typename T>
__device__ void xsolid_j2(const XSolid& S, int e, double ak, double am) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1, NS = ND == 2 ? 3 : 6;
    const int32_t* ed = S.edof + (size_t)e * NC;
    T u1[NC], u2[NC], y[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const int t = ed[j];
        u1[j] = (T)(S.xK ? S.xK[t] : 0.0);
        u2[j] = (T)((S.xK2 && S.cK2 != 0.0) ? S.cK2 * ak * S.xK2[t] : 0.0);
        y[j] = 0.0;
    }
    const T c1 = (T)S.coef[3 * e], c2 = (T)S.coef[3 * e + 1], c3 = (T)S.coef[3 * e + 2];
    const double* g0 = S.geo + (size_t)S.egeo[e] * S.ngp * PER;
    const size_t cs = (size_t)S.ngp * S.n;
    for (int q = 0; q < S.ngp; ++q) {
        const double* g = g0 + q * PER;
        T b[NEN][3];
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[a][j] = (T)((j < ND) ? g[a * ND + j] : 0.0);
        const T w = (T)g[PER - 1];
        T e1[6], e2[6], sig[6];
        xstrain<ND, NEN, T>(b, u1, e1);
        xstrain<ND, NEN, T>(b, u2, e2);
        xelastic<ND, T>(c1, c2, c3, e2, sig);
        const double* ct = S.ctan + (size_t)q * S.n + e;
#pragma unroll
        for (int a = 0; a < NS; ++a) {
            T v = 0;
#pragma unroll
            for (int bb = 0; bb < NS; ++bb) v += (T)ct[(size_t)(a * NS + bb) * cs] * e1[bb];
            sig[a] += v;
        }
        xbts<ND, NEN, T>(b, w, sig, y);
    }
    if (S.xM || S.xM2) {
        const double* ml = S.mlump + (size_t)e * NEN;
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            const int t = ed[j];
            double v = S.xM ? S.sM * S.xM[t] : 0.0;
            if (S.xM2 && S.cM2 != 0.0) v += S.cM2 * am * S.xM2[t];
            y[j] += (T)(ml[j / ND] * v);
        }
    }
    double* out = S.y + (size_t)e * NC;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        double v = (double)y[j];
        if (S.ftol >= 0.0 && !(fabs(v) > S.ftol)) v = 0.0;
        v *= S.yscale;
        out[j] = S.accumulate ? out[j] + v : v;
    }
}

// Element::UpdateState from the strain displacement Us for every solid
// element (elastic: sigma = C eps; J2: the return mapping in place on the
// Gauss-point state, storing the consistent tangent), then the internal force
// B^T sigma with the assembler's force tolerance (Assembler.cpp:262).
struct XState {
    int n, ngp;
    const int32_t* edof; const int32_t* egeo; const double* geo; const double* coef;
    const int32_t* kind;     // [n] or null
    const double* j2p;       // [n][5] K G H beta SY
    double* state;           // [13][ngp][n]
    double* ctan;            // [NS*NS][ngp][n]
    float* ctan_f;           // [NS*NS][ngp][n] single-precision copy, or null
    const double* Us;
    double ftol;
    double* fint;            // [n][NC]
};

template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_xstate(XState S) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= S.n) return;
    const int32_t* ed = S.edof + (size_t)e * NC;
    double ue[NC], fe[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) { ue[j] = S.Us[ed[j]]; fe[j] = 0.0; }
    const bool j2 = S.kind && S.kind[e];
    const double c1 = S.coef[3 * e], c2 = S.coef[3 * e + 1], c3 = S.coef[3 * e + 2];
    const double* g0 = S.geo + (size_t)S.egeo[e] * S.ngp * PER;
    const size_t gs = (size_t)S.ngp * S.n;
    for (int q = 0; q < S.ngp; ++q) {
        const double* g = g0 + q * PER;
        double b[NEN][3];
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[a][j] = (j < ND) ? g[a * ND + j] : 0.0;
        const double w = g[PER - 1];
        double ev[6], sig[6];
        xstrain<ND, NEN, double>(b, ue, ev);
        if (!j2) {
            xelastic<ND, double>(c1, c2, c3, ev, sig);
        } else {
            const double* p = S.j2p + (size_t)e * 5;
            double st[kJ2State];
            double* sp = S.state + (size_t)q * S.n + e;
#pragma unroll
            for (int i = 0; i < kJ2State; ++i) st[i] = sp[(size_t)i * gs];
            double s6[6];
            if (ND == 2) {
                const double Ev[6] = {0.0, ev[0], ev[1], 0.0, 0.5 * ev[2], 0.0};
                j2_return<2>(Ev, st, p[0], p[1], p[2], p[3], p[4], s6, S.ctan + (size_t)q * S.n + e, gs);
                sig[0] = s6[1]; sig[1] = s6[2]; sig[2] = s6[4];
                sig[3] = sig[4] = sig[5] = 0.0;
            } else {
                const double Ev[6] = {ev[0], ev[1], ev[2], 0.5 * ev[3], 0.5 * ev[4], 0.5 * ev[5]};
                j2_return<3>(Ev, st, p[0], p[1], p[2], p[3], p[4], s6, S.ctan + (size_t)q * S.n + e, gs);
#pragma unroll
                for (int i = 0; i < 6; ++i) sig[i] = s6[i];
            }
            if (S.ctan_f) {
                constexpr int NS = ND == 2 ? 3 : 6;
                const double* ct = S.ctan + (size_t)q * S.n + e;
                float* cf = S.ctan_f + (size_t)q * S.n + e;
#pragma unroll
                for (int i = 0; i < NS * NS; ++i) cf[(size_t)i * gs] = (float)ct[(size_t)i * gs];
            }
#pragma unroll
            for (int i = 0; i < kJ2State; ++i) sp[(size_t)i * gs] = st[i];
        }
        xbts<ND, NEN, double>(b, w, sig, fe);
    }
    double* out = S.fint + (size_t)e * NC;
#pragma unroll
    for (int j = 0; j < NC; ++j) out[j] = (fabs(fe[j]) > S.ftol) ? fe[j] : 0.0;
}

__global__ void k_xneg(size_t n, const double* __restrict__ a, double* __restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = -a[i];
}

// T = double, or float for the inner solver iterations (see k_pml_action)
template <int ND, int NEN, typename T>
__global__ void __launch_bounds__(128) k_xsolid(XSolid S) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= S.n) return;
    const int32_t* ed = S.edof + (size_t)e * NC;
    const double am = S.ray ? S.ray[2 * e] : 0.0, ak = S.ray ? S.ray[2 * e + 1] : 0.0;
    if (S.kind && S.kind[e]) {
        xsolid_j2<ND, NEN, T>(S, e, ak, am);
        return;
    }
    T uk[NC], y[NC];
    // an operator application passes one vector for every input: load it once
    const bool one = S.xK && S.xK2 == S.xK && S.xM == S.xK && S.xM2 == S.xK;
    double pm[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const int t = ed[j];
        double v;
        if (one) {
            const double p = S.xK[t];
            pm[j] = p;
            v = p;
            if (S.cK2 != 0.0) v += S.cK2 * ak * p;
        } else {
            v = S.xK ? S.xK[t] : 0.0;
            if (S.xK2 && S.cK2 != 0.0) v += S.cK2 * ak * S.xK2[t];
        }
        uk[j] = (T)v;
        y[j] = 0;
    }
    const T c1 = (T)S.coef[3 * e], c2 = (T)S.coef[3 * e + 1], c3 = (T)S.coef[3 * e + 2];
    const double* g0 = S.geo + (size_t)S.egeo[e] * S.ngp * PER;
    for (int q = 0; q < S.ngp; ++q) {
        const double* g = g0 + q * PER;
        T b[NEN][3];
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[a][j] = (T)((j < ND) ? g[a * ND + j] : 0.0);
        const T w = (T)g[PER - 1];
        if (ND == 2) {
            T exx = 0, eyy = 0, gxy = 0;
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                exx += b[a][0] * uk[2 * a];
                eyy += b[a][1] * uk[2 * a + 1];
                gxy += b[a][1] * uk[2 * a] + b[a][0] * uk[2 * a + 1];
            }
            const T s0 = c1 * exx + c2 * eyy, s1 = c2 * exx + c1 * eyy, s2 = c3 * gxy;
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                y[2 * a] += w * (b[a][0] * s0 + b[a][1] * s2);
                y[2 * a + 1] += w * (b[a][1] * s1 + b[a][0] * s2);
            }
        } else {
            T ev[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                const T ux = uk[3 * a], uy = uk[3 * a + 1], uz = uk[3 * a + 2];
                ev[0] += b[a][0] * ux;
                ev[1] += b[a][1] * uy;
                ev[2] += b[a][2] * uz;
                ev[3] += b[a][1] * ux + b[a][0] * uy;
                ev[4] += b[a][2] * uy + b[a][1] * uz;
                ev[5] += b[a][2] * ux + b[a][0] * uz;
            }
            T sg[6];
            sg[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
            sg[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
            sg[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
            sg[3] = c3 * ev[3]; sg[4] = c3 * ev[4]; sg[5] = c3 * ev[5];
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                const T bx = b[a][0], by = b[a][1], bz = b[a][2];
                y[3 * a] += w * (bx * sg[0] + by * sg[3] + bz * sg[5]);
                y[3 * a + 1] += w * (by * sg[1] + bx * sg[3] + bz * sg[4]);
                y[3 * a + 2] += w * (bz * sg[2] + by * sg[4] + bx * sg[5]);
            }
        }
    }
    if (S.xM || S.xM2) {
        const double* ml = S.mlump + (size_t)e * NEN;
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            double v;
            if (one) {
                v = S.sM * pm[j];
                if (S.cM2 != 0.0) v += S.cM2 * am * pm[j];
            } else {
                const int t = ed[j];
                v = S.xM ? S.sM * S.xM[t] : 0.0;
                if (S.xM2 && S.cM2 != 0.0) v += S.cM2 * am * S.xM2[t];
            }
            y[j] += (T)(ml[j / ND] * v);
        }
    }
    double* out = S.y + (size_t)e * NC;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        double v = (double)y[j];
        if (S.ftol >= 0.0 && !(fabs(v) > S.ftol)) v = 0.0;
        v *= S.yscale;
        out[j] = S.accumulate ? out[j] + v : v;
    }
}

// Operator action y_e = (K_e + cK2 ak_e K0_e + sM M_e + cM2 am_e M_e) p_e with
// one thread per (element, Gauss point): the NEN (= number of Gauss points)
// threads of an element are consecutive lanes of a warp, lane q loads node
// q's dofs, the element vector reaches the other lanes by shuffles, each lane
// forms its Gauss point's w B^T sigma and a butterfly over the NEN lanes sums
// them; lane q adds node q's lumped mass term and writes node q's entries.
// Eight times the threads of k_xsolid at about a third of its registers: the
// element-per-thread form is bound by load latency at low occupancy.
template <int ND, int NEN, typename T>
__global__ void __launch_bounds__(128) k_xsolid_gp(XSolid S) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1, NS = ND == 2 ? 3 : 6;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int e = gtid / NEN, q = gtid % NEN;
    const bool valid = e < S.n;
    const int ec = valid ? e : S.n - 1;
    const int lane = threadIdx.x & 31, base = lane - q;
    const int32_t* ed = S.edof + (size_t)ec * NC;
    const bool j2 = S.kind && S.kind[ec];
    double pq[ND];
    T pt[ND];
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
        for (int c = 0; c < ND; ++c) { pt[c] = S.xK_f[ed[q * ND + c]]; pq[c] = 0.0; }
    } else {
#pragma unroll
        for (int c = 0; c < ND; ++c) { pq[c] = S.xK[ed[q * ND + c]]; pt[c] = pq[c]; }
    }
    double am = 0.0;
    T kscale, c1, c2, c3;                      // kscale: stiffness-proportional damping factor
    if constexpr (std::is_same<T, float>::value) {
        const float* o = S.opf + (size_t)ec * (NEN + 4);
        kscale = o[NEN]; c1 = o[NEN + 1]; c2 = o[NEN + 2]; c3 = o[NEN + 3];
    } else {
        am = S.ray ? S.ray[2 * ec] : 0.0;
        const double ak = S.ray ? S.ray[2 * ec + 1] : 0.0;
        kscale = S.cK2 != 0.0 ? S.cK2 * ak : 0.0;
        c1 = S.coef[3 * ec]; c2 = S.coef[3 * ec + 1]; c3 = S.coef[3 * ec + 2];
    }
    T b[NEN][3], w;
    if constexpr (std::is_same<T, float>::value) {
        const float* g = S.geo_f + ((size_t)S.egeo[ec] * S.ngp + q) * PER;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[a][j] = (j < ND) ? g[a * ND + j] : 0.0f;
        w = g[PER - 1];
    } else {
        const double* g = S.geo + ((size_t)S.egeo[ec] * S.ngp + q) * PER;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) b[a][j] = (j < ND) ? g[a * ND + j] : 0.0;
        w = g[PER - 1];
    }
    // strain of p at this Gauss point
    T ev[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
        T ua[3] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < ND; ++c) ua[c] = __shfl_sync(0xffffffffu, pt[c], base + a);
        if (ND == 2) {
            ev[0] += b[a][0] * ua[0];
            ev[1] += b[a][1] * ua[1];
            ev[2] += b[a][1] * ua[0] + b[a][0] * ua[1];
        } else {
            ev[0] += b[a][0] * ua[0];
            ev[1] += b[a][1] * ua[1];
            ev[2] += b[a][2] * ua[2];
            ev[3] += b[a][1] * ua[0] + b[a][0] * ua[1];
            ev[4] += b[a][2] * ua[1] + b[a][1] * ua[2];
            ev[5] += b[a][2] * ua[0] + b[a][0] * ua[2];
        }
    }
    T sig[6];
    xelastic<ND, T>(c1, c2, c3, ev, sig);
    if (j2) {
        // tangent on p plus the initial elastic tangent on kscale p
        const size_t cs = (size_t)S.ngp * S.n;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            T v = 0;
#pragma unroll
            for (int jj = 0; jj < NS; ++jj) {
                T c;
                if constexpr (std::is_same<T, float>::value) c = S.ctan_f[(size_t)(i * NS + jj) * cs + (size_t)q * S.n + ec];
                else c = S.ctan[(size_t)(i * NS + jj) * cs + (size_t)q * S.n + ec];
                v += c * ev[jj];
            }
            sig[i] = kscale * sig[i] + v;
        }
    } else {
#pragma unroll
        for (int i = 0; i < NS; ++i) sig[i] *= (T(1.0) + kscale);
    }
    T y[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) y[j] = 0;
    xbts<ND, NEN, T>(b, w, sig, y);
#pragma unroll
    for (int off = 1; off < NEN; off <<= 1)
#pragma unroll
        for (int j = 0; j < NC; ++j) y[j] += __shfl_xor_sync(0xffffffffu, y[j], off);
    if (!valid) return;
    if constexpr (std::is_same<T, float>::value) {
        // single precision: mass term from the table, float element vector
        const float mmf = S.opf[(size_t)ec * (NEN + 4) + q];
        float* outf = S.y_f + (size_t)ec * NC + q * ND;
#pragma unroll
        for (int c = 0; c < ND; ++c) {
            T mine = 0;
#pragma unroll
            for (int a = 0; a < NEN; ++a)
                if (a == q) mine = y[a * ND + c];
            outf[c] = mine + mmf * pt[c];
        }
        return;
    }
    double* out = S.y + (size_t)ec * NC + q * ND;
    const double ml = S.mlump[(size_t)ec * NEN + q];
#pragma unroll
    for (int c = 0; c < ND; ++c) {
        T mine = 0;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
            if (a == q) mine = y[a * ND + c];
        double v = (double)mine;
        {
            double mv = S.sM * pq[c];
            if (S.cM2 != 0.0) mv += S.cM2 * am * pq[c];
            v += ml * mv;
        }
        if (S.ftol >= 0.0 && !(fabs(v) > S.ftol)) v = 0.0;
        v *= S.yscale;
        out[c] = S.accumulate ? out[c] + v : v;
    }
}

// Domain-reduction forces (lin2DQuad4.cpp:564-614) of solid elastic elements
// with a lumped mass: factor * K~ (U_o + ak V_o), K~ coupling only boundary and
// exterior dofs (see k_drm in svl_cd.cu for the same reduction).
struct XDrm {
    int n, nt, k, ngp;
    const int32_t* sidx;      // [n] solid-element index of each entry
    const double* factor;     // [n]
    const double* ak;         // [n]
    const int32_t* node_of;   // [n][NEN]
    const int32_t* row;       // [nnode]
    const int32_t* ext;       // [nnode]
    const double* motion;     // [blocks][nt][3 ND]
    const int32_t* egeo; const double* geo; const double* coef;
    double* fe;               // [n][NC]
};

template <int ND, int NEN>
__global__ void __launch_bounds__(128) k_xdrm(XDrm D) {
    constexpr int NC = ND * NEN, PER = NEN * ND + 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.n) return;
    const int e = D.sidx[i], k = D.k;
    double wb[NC], we[NC], yb[NC], ye[NC];
    int ext[NEN];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const int a = j / ND, c = j % ND;
        const int node = D.node_of[(size_t)i * NEN + a];
        const bool x = D.ext[node] != 0;
        ext[a] = x;
        double u = 0.0, v = 0.0;
        if (k >= 0 && k < D.nt) {
            const double* rw = D.motion + ((size_t)D.row[node] * D.nt + k) * (3 * ND);
            u = rw[c];
            v = rw[ND + c];
        }
        const double w = (x ? -1.0 : 1.0) * (u + D.ak[i] * v);
        wb[j] = x ? 0.0 : w;
        we[j] = x ? w : 0.0;
        yb[j] = 0.0; ye[j] = 0.0;
    }
    const double c1 = D.coef[3 * e], c2 = D.coef[3 * e + 1], c3 = D.coef[3 * e + 2];
    const double* g0 = D.geo + (size_t)D.egeo[e] * D.ngp * PER;
    for (int q = 0; q < D.ngp; ++q) {
        const double* g = g0 + q * PER;
        const double w = g[PER - 1];
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
            const double* uu = pass == 0 ? wb : we;
            double* yy = pass == 0 ? yb : ye;
            if (ND == 2) {
                double exx = 0, eyy = 0, gxy = 0;
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    const double bx = g[a * ND], by = g[a * ND + 1];
                    exx += bx * uu[2 * a];
                    eyy += by * uu[2 * a + 1];
                    gxy += by * uu[2 * a] + bx * uu[2 * a + 1];
                }
                const double s0 = c1 * exx + c2 * eyy, s1 = c2 * exx + c1 * eyy, s2 = c3 * gxy;
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    const double bx = g[a * ND], by = g[a * ND + 1];
                    yy[2 * a] += w * (bx * s0 + by * s2);
                    yy[2 * a + 1] += w * (by * s1 + bx * s2);
                }
            } else {
                double ev[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    const double bx = g[a * ND], by = g[a * ND + 1], bz = g[a * ND + (ND - 1)];
                    const double ux = uu[ND * a], uy = uu[ND * a + 1], uz = uu[ND * a + (ND - 1)];
                    ev[0] += bx * ux;
                    ev[1] += by * uy;
                    ev[2] += bz * uz;
                    ev[3] += by * ux + bx * uy;
                    ev[4] += bz * uy + by * uz;
                    ev[5] += bz * ux + bx * uz;
                }
                double sg[6];
                sg[0] = c1 * ev[0] + c2 * ev[1] + c2 * ev[2];
                sg[1] = c2 * ev[0] + c1 * ev[1] + c2 * ev[2];
                sg[2] = c2 * ev[0] + c2 * ev[1] + c1 * ev[2];
                sg[3] = c3 * ev[3]; sg[4] = c3 * ev[4]; sg[5] = c3 * ev[5];
#pragma unroll
                for (int a = 0; a < NEN; ++a) {
                    const double bx = g[a * ND], by = g[a * ND + 1], bz = g[a * ND + (ND - 1)];
                    yy[ND * a] += w * (bx * sg[0] + by * sg[3] + bz * sg[5]);
                    yy[ND * a + 1] += w * (by * sg[1] + bx * sg[3] + bz * sg[4]);
                    yy[ND * a + (ND - 1)] += w * (bz * sg[2] + by * sg[4] + bx * sg[5]);
                }
            }
        }
    }
    double* out = D.fe + (size_t)i * NC;
#pragma unroll
    for (int j = 0; j < NC; ++j) out[j] = D.factor[i] * (ext[j / ND] ? yb[j] : ye[j]);
}

// y_t = sum of the element entries of dof t in element order (+ c_n m_t x_t) (+ Fext_t(k))
struct XGather {
    int ntotal;
    const int64_t* inv_ptr;      // [ntotal+1]
    const int64_t* inv_idx;      // into fe (solid block, then PML block)
    const double* fe;
    const double* nodemass;      // [ntotal] or null
    double cn;
    const double* xn;
    // Lysmer dashpots: + cdp sum eta (x_t - x_partner)
    const int32_t *dp_ptr, *dp_col; const double* dp_eta;
    double cdp;
    const double* xdp;
    // external force (RHS only), with the domain-reduction element forces
    int k, with_fext;
    const int32_t *drm_ptr, *drm_idx; const double* drm_fe;
    const int32_t *ld_ptr, *ld_ser; const double* ld_coef;
    const int32_t* s_ptr; const double* s_val;
    double* y;
};

__global__ void k_xgather(XGather G) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G.ntotal) return;
    double v = 0.0;
    for (int64_t i = G.inv_ptr[t]; i < G.inv_ptr[t + 1]; ++i) v += G.fe[G.inv_idx[i]];
    if (G.nodemass && G.xn) v += G.cn * G.nodemass[t] * G.xn[t];
    if (G.dp_ptr && G.xdp) {
        double c = 0.0;
        const double xt = G.xdp[t];
        for (int i = G.dp_ptr[t]; i < G.dp_ptr[t + 1]; ++i) c += G.dp_eta[i] * (xt - G.xdp[G.dp_col[i]]);
        v += G.cdp * c;
    }
    if (G.with_fext) {
        double f = 0.0;
        for (int i = G.ld_ptr[t]; i < G.ld_ptr[t + 1]; ++i) {
            const int s = G.ld_ser[i];
            const int b = G.s_ptr[s], n = G.s_ptr[s + 1] - b;
            f += G.ld_coef[i] * ((G.k >= 0 && G.k < n) ? G.s_val[b + G.k] : 0.0);
        }
        if (G.drm_ptr)
            for (int i = G.drm_ptr[t]; i < G.drm_ptr[t + 1]; ++i) f += G.drm_fe[G.drm_idx[i]];
        v += f;
    }
    G.y[t] = v;
}

// out_t = sum_f T_tf x_f
__global__ void k_xexpand(int ntotal, const int32_t* __restrict__ Tp, const int32_t* __restrict__ Tc,
                          const double* __restrict__ Tv, const double* __restrict__ x, double* __restrict__ out,
                          float* __restrict__ out_f = nullptr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntotal) return;
    double v = 0.0;
    for (int i = Tp[t]; i < Tp[t + 1]; ++i) v += Tv[i] * x[Tc[i]];
    out[t] = v;
    if (out_f) out_f[t] = (float)v;
}

// y_t = sum of the float element entries of dof t in element order (summed in
// float, converted once) + cn m_t x_t + cdp sum eta (x_t - x_partner): the
// gather of the single-precision operator
__global__ void k_xgather_f(int ntotal, const int64_t* __restrict__ inv_ptr, const int64_t* __restrict__ inv_idx,
                            const float* __restrict__ fe, const double* nodemass, double cn, const double* xn,
                            const int32_t* dp_ptr, const int32_t* dp_col, const double* dp_eta, double cdp,
                            const double* xdp, double* __restrict__ y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntotal) return;
    float vf = 0.0f;
    for (int64_t i = inv_ptr[t]; i < inv_ptr[t + 1]; ++i) vf += fe[inv_idx[i]];
    double v = (double)vf;
    if (nodemass) v += cn * nodemass[t] * xn[t];
    if (dp_ptr && dp_ptr[t + 1] > dp_ptr[t]) {
        double c = 0.0;
        const double xt = xdp[t];
        for (int i = dp_ptr[t]; i < dp_ptr[t + 1]; ++i) c += dp_eta[i] * (xt - xdp[dp_col[i]]);
        v += cdp * c;
    }
    y[t] = v;
}

// out_f = sum_t T_tf y_t (- sum_t T_tf z_t)
__global__ void k_xreduce(int nfree, const int32_t* __restrict__ TTp, const int32_t* __restrict__ TTr,
                          const double* __restrict__ TTv, const double* __restrict__ y, const double* __restrict__ z,
                          double* __restrict__ out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfree) return;
    double v = 0.0, w = 0.0;
    for (int i = TTp[f]; i < TTp[f + 1]; ++i) {
        v += TTv[i] * y[TTr[i]];
        if (z) w += TTv[i] * z[TTr[i]];
    }
    out[f] = z ? v - w : v;
}

// support-motion increment of step k on total dofs (Assembler.cpp:493-532)
__global__ void k_xsm(int ntotal, const int32_t* sm_ptr, const int32_t* sm_ser, const double* sm_fac,
                      const int32_t* s_ptr, const double* s_val, int k, double* sm) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntotal) return;
    double v = 0.0;
    for (int i = sm_ptr[t]; i < sm_ptr[t + 1]; ++i) {
        const int s = sm_ser[i];
        const int b = s_ptr[s], n = s_ptr[s + 1] - b;
        double g = 0.0;
        if (n > 0) {
            g = (k >= 0 && k < n) ? s_val[b + k] : s_val[b];
            if (k > 0) g -= (k - 1 < n ? s_val[b + k - 1] : s_val[b]);
        }
        v += sm_fac[i] * g;
    }
    sm[t] = v;
}

// W = 4/dt V + A and Wg = Ubar + dt U + dt^2/6 V
__global__ void k_xrhs_vec(int n, const double* U, const double* V, const double* A, const double* Ub, double dt,
                           double* W, double* Wg) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    W[t] = 4.0 / dt * V[t] + A[t];
    Wg[t] = Ub[t] + dt * U[t] + dt * dt / 6.0 * V[t];
}

// NewmarkBeta: W = 4/dt V + A - 4/dt^2 dU and Vd = V - 2/dt dU (NewmarkBeta.cpp:215)
__global__ void k_xrhs_nm(int n, const double* V, const double* A, const double* dUt, double dt, double* W,
                          double* Vd) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    W[t] = 4.0 / dt * V[t] + A[t] - 4.0 / dt / dt * dUt[t];
    Vd[t] = V[t] - 2.0 / dt * dUt[t];
}

// ExtendedNewmarkBeta::ComputeNewStep state update (dUt = T du, sm = SM(k));
// NewmarkBeta's (no PML history) with pml_hist = 0
__global__ void k_xupdate(int n, double* U, double* V, double* A, double* Ub, double* Us, const double* dUt,
                          const double* sm, double dt, int pml_hist, int* bad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double d = dUt[t], D = d + (sm ? sm[t] : 0.0);
    const double u = U[t], v = V[t];
    if (pml_hist) Ub[t] = Ub[t] + dt * u + dt / 3.0 * D + dt * dt / 6.0 * v;
    Us[t] = u + d;                       // solid strain displacement: U + T du
    const double un = u + D;
    U[t] = un;
    A[t] = 4.0 / dt / dt * d - 4.0 / dt * v - A[t];
    V[t] = 2.0 / dt * d - v;
    if (!isfinite(un)) atomicOr(bad, 1);
}

__global__ void k_xdot_partial(const double* __restrict__ a, const double* __restrict__ b, int n, double* partial) {
    __shared__ double sh[kThreads / 32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += a[i] * b[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}
__global__ void k_xdot_final(const double* __restrict__ partial, double* out) {
    __shared__ double sh[kThreads / 32];
    double s = 0.0;
    for (int i = threadIdx.x; i < kBlocks; i += kThreads) s += partial[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) *out = v;
    }
}

__global__ void k_xadd(int n, const double* a, const double* b, double* out) {       // out = a + b
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] + b[i];
}
__global__ void k_xaxpby(int n, double a, const double* x, double b, double* y) {   // y = a x + b y
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = a * x[i] + b * y[i];
}
__global__ void k_xvmul(int n, const double* a, const double* b, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] * b[i];
}
__global__ void k_xsub(int n, const double* a, const double* b, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}
// MINRES direction and iterate: w = (v - oldeps w1 - delta w2) / gamma; x += phi w
// R_t = -y_t on the dofs of fixed nodes, 0 elsewhere (Node::GetReaction)
__global__ void k_xreact(int n, const int8_t* __restrict__ fixed, const double* __restrict__ y, double* __restrict__ R) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) R[t] = fixed[t] ? -y[t] : 0.0;
}
__global__ void k_xmr_w(int n, const double* v, const double* w1, const double* w2, double* w, double* x,
                        double oldeps, double delta, double inv_gamma, double phi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double wi = (v[i] - oldeps * w1[i] - delta * w2[i]) * inv_gamma;
    w[i] = wi;
    x[i] += phi * wi;
}
// unit vector e_i in every element block (diagonal probes)
__global__ void k_xunit(int nel, int nc, int i, double* u) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (int64_t)nel * nc) return;
    u[j] = (j % nc) == i ? 1.0 : 0.0;
}
__global__ void k_xtake(int nel, int nc, int i, const double* y, double* d) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nel) d[(size_t)e * nc + i] = y[(size_t)e * nc + i];
}

// ---- explicit central difference with PML layers (integrator
// SVL_XNM_CENTRAL_DIFFERENCE).  A scheme of this library: the reference's
// CentralDifference applies no PML history and keeps the PML mass consistent
// and indefinite (CentralDifference.cpp:114-120, PML3DHexa8.cpp:214-284).
// Displacements live at the integer steps, the PML stress dofs S at the half
// steps; the N N blocks of the PML element matrices are row-sum lumped per
// node (a diagonal on displacement dofs, an ns x ns block on a node's stress
// dofs) and the displacement-stress couplings act through the element action
// (svl_pml.cu) on vectors whose other class of dofs is zero.

// inputs of the displacement rows: on stress dofs sdot = (S - Sp)/dt,
// smid = (S + Sp)/2 and Sbar; zero on displacement dofs
__global__ void k_cdp_sin(int n, const int8_t* __restrict__ sdof, const double* __restrict__ U,
                          const double* __restrict__ Up, const double* __restrict__ Ub, double dt,
                          double* __restrict__ x0, double* __restrict__ x1, double* __restrict__ x2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (sdof[t]) {
        x0[t] = (U[t] - Up[t]) / dt;
        x1[t] = (U[t] + Up[t]) / 2.0;
        x2[t] = Ub[t];
    } else {
        x0[t] = 0.0; x1[t] = 0.0; x2[t] = 0.0;
    }
}

// displacement rows: R = (y - Ku u - Gu ubar) + (Mu/dt^2 - Cu/2dt)(u - up),
// y = Fext(k) - (solid internal force + couplings): the increment form of
// the plain central difference (CentralDifference.cpp:206-221) with the
// lumped PML terms; zero on stress dofs
__global__ void k_cdp_r(int n, const int8_t* __restrict__ sdof, const double* __restrict__ y,
                        const double* __restrict__ Mu, const double* __restrict__ Cu, const double* __restrict__ Ku,
                        const double* __restrict__ Gu, double dt, const double* __restrict__ U,
                        const double* __restrict__ Up, const double* __restrict__ Ub, double* __restrict__ R) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (sdof[t]) { R[t] = 0.0; return; }
    const double c = 1.0 / dt / dt * Mu[t] - 1.0 / 2.0 / dt * Cu[t];
    R[t] = (y[t] - Ku[t] * U[t] - Gu[t] * Ub[t]) + c * (U[t] - Up[t]);
}

// the diagonal solve of T^T (Mu/dt^2 + Cu/2dt) T as (1/d) b (0 on stress dofs)
__global__ void k_cdp_solve(int nf, const double* __restrict__ kinv, const double* __restrict__ b, double* __restrict__ x) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    x[f] = kinv[f] * b[f];
}

// displacement increment dUt = T du (+ the support-motion increment), the
// trapezoid ubar, the solid strain displacement U + T du, and the inputs of
// the stress rows (udot, umid, ubar at the half step; zero on stress dofs)
__global__ void k_cdp_u(int n, const int8_t* __restrict__ sdof, const double* __restrict__ dUt,
                        const double* __restrict__ sm, double dt, const double* __restrict__ U,
                        const double* __restrict__ Ub, double* __restrict__ dU, double* __restrict__ Us,
                        double* __restrict__ Ubn, double* __restrict__ x0, double* __restrict__ x1,
                        double* __restrict__ x2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (sdof[t]) { x0[t] = 0.0; x1[t] = 0.0; x2[t] = 0.0; return; }
    const double u = U[t], du = dUt[t];
    Us[t] = u + du;                                  // strain without the support-motion increment
    const double D = du + (sm ? sm[t] : 0.0);
    dU[t] = D;
    const double un = u + D;
    const double ubn = Ub[t] + dt * (u + un) / 2.0;
    Ubn[t] = ubn;
    x0[t] = (un - u) / dt;
    x1[t] = (un + u) / 2.0;
    x2[t] = (Ub[t] + ubn) / 2.0;
}

// stress rows of PML node i: (Ms/dt^2 + Cs/2dt) dS = -Fs - Ks S - Gs Sbar_half
// + (Ms/dt^2 - Cs/2dt)(S - Sp), solved with the stored inverse
template <int NS>
__global__ void k_cdp_s(int nsn, const int32_t* __restrict__ sfirst, const double* __restrict__ Fs,
                        const double* __restrict__ Ms, const double* __restrict__ Cs, const double* __restrict__ Ks,
                        const double* __restrict__ Gs, const double* __restrict__ Dinv, const double* __restrict__ U,
                        const double* __restrict__ Up, const double* __restrict__ Ub, double dt,
                        double* __restrict__ dU, double* __restrict__ Ubn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nsn) return;
    const int t0 = sfirst[i];
    const size_t b = (size_t)i * NS * NS;
    double sc[NS], sp[NS], sbh[NS], R[NS];
#pragma unroll
    for (int c = 0; c < NS; ++c) {
        sc[c] = U[t0 + c]; sp[c] = Up[t0 + c];
        sbh[c] = Ub[t0 + c] + dt / 2.0 * sc[c];
    }
#pragma unroll
    for (int r = 0; r < NS; ++r) {
        double v = -Fs[t0 + r];
#pragma unroll
        for (int c = 0; c < NS; ++c) {
            const size_t k = b + r * NS + c;
            v += -Ks[k] * sc[c] - Gs[k] * sbh[c] + (Ms[k] / dt / dt - Cs[k] / 2.0 / dt) * (sc[c] - sp[c]);
        }
        R[r] = v;
    }
#pragma unroll
    for (int r = 0; r < NS; ++r) {
        double v = 0.0;
#pragma unroll
        for (int c = 0; c < NS; ++c) v += Dinv[b + r * NS + c] * R[c];
        dU[t0 + r] = v;
        Ubn[t0 + r] = Ub[t0 + r] + dt * sc[r];
    }
}

// CentralDifference::ComputeNewStep's update on every dof (:138-148)
__global__ void k_cdp_update(int n, double* __restrict__ U, double* __restrict__ Up, double* __restrict__ V,
                             double* __restrict__ A, double* __restrict__ Ub, const double* __restrict__ dU,
                             const double* __restrict__ Ubn, double dt, int* bad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double u = U[t], d = dU[t], up = Up[t];
    V[t] = 1.0 / 2.0 / dt * (u + d - up);
    A[t] = 1.0 / dt / dt * (d - u + up);
    Up[t] = u;
    const double un = u + d;
    U[t] = un;
    Ub[t] = Ubn[t];
    if (!isfinite(un)) atomicOr(bad, 1);
}

// Up = U - dt V + dt^2/2 A (CentralDifference.cpp:61)
__global__ void k_cdp_init(int n, const double* U, const double* V, const double* A, double dt, double* Up) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    Up[t] = U[t] - dt * V[t] + dt * dt / 2.0 * A[t];
}

}  // namespace

struct svl_xnm {
    HostModel m;
    svl_xnm_opts opts{};
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    int nsol = 0, npml = 0, ncs = 0, ncp = 0;
    // solid elements
    int32_t *s_edof = nullptr, *s_egeo = nullptr, *s_kind = nullptr;
    double *s_geo = nullptr, *s_coef = nullptr, *s_ray = nullptr, *s_mlump = nullptr;
    double *s_j2p = nullptr, *s_state = nullptr, *s_ctan = nullptr, *s_fint = nullptr;
    float *s_geo_f = nullptr, *s_ctan_f = nullptr;   // single-precision copies
    float* s_opf = nullptr;                           // [nsol][nen + 4] (XSolid::opf)
    bool has_j2 = false, newton = false;
    // PML elements
    double *p_X = nullptr, *p_mat = nullptr, *p_thick = nullptr, *p_par = nullptr;
    float* p_tab = nullptr;                  // single-precision element constants
    int32_t* p_edof = nullptr;
    // element vectors and their ordered gather
    double* fe = nullptr;
    int64_t *inv_ptr = nullptr, *inv_idx = nullptr;
    double* nodemass = nullptr;
    int32_t *dp_ptr = nullptr, *dp_col = nullptr;
    double* dp_eta = nullptr;
    // domain reduction
    int ndrm = 0, drm_nt = 0;
    int32_t *drm_sidx = nullptr, *drm_node_of = nullptr, *drm_row = nullptr, *drm_ext = nullptr;
    int32_t *drm_ptr = nullptr, *drm_idx = nullptr;
    double *drm_factor = nullptr, *drm_ak = nullptr, *drm_motion = nullptr, *drm_fe = nullptr;
    // T and T^T
    int32_t *Tp = nullptr, *Tc = nullptr, *TTp = nullptr, *TTr = nullptr;
    double *Tv = nullptr, *TTv = nullptr;
    // loads
    LoadTables lt;
    int32_t *ld_ptr = nullptr, *ld_ser = nullptr, *s_ptr = nullptr, *sm_ptr = nullptr, *sm_ser = nullptr;
    double *ld_coef = nullptr, *s_val = nullptr, *sm_fac = nullptr;
    // state (total dofs) and scratch
    double *U = nullptr, *V = nullptr, *A = nullptr, *Ub = nullptr, *Us = nullptr;
    double *W = nullptr, *Wg = nullptr, *yt = nullptr, *ys = nullptr, *pt = nullptr, *sm = nullptr, *dUt = nullptr;
    double* Ui = nullptr;                    // U + T dU: the PML elements' displacement
    float *pt_f = nullptr, *fe_f = nullptr;  // single-precision operator input and element vectors
    bool newmark = false;                    // NewmarkBeta instead of ExtendedNewmarkBeta
    bool explicit_cd = false;                // explicit central difference with PML (staggered scheme)
    // explicit scheme: lumped diagonals of the displacement rows, stress dofs,
    // per-PML-node stress blocks, previous state and the half-step integrals
    int8_t* cd_sdof = nullptr;
    double *cd_Mu = nullptr, *cd_Cu = nullptr, *cd_Ku = nullptr, *cd_Gu = nullptr;
    int cd_nsn = 0;
    int32_t* cd_sfirst = nullptr;
    double *cd_Ms = nullptr, *cd_Cs = nullptr, *cd_Ks = nullptr, *cd_Gs = nullptr, *cd_Dinv = nullptr;
    double *cd_Up = nullptr, *cd_Ubn = nullptr, *cd_kinv = nullptr;
    // free-dof vectors
    double *b = nullptr, *x = nullptr, *dUf = nullptr, *r1 = nullptr, *r2 = nullptr, *yv = nullptr, *v = nullptr;
    double *w = nullptr, *w1 = nullptr, *w2 = nullptr, *dinv = nullptr, *tmp = nullptr;
    double *partial = nullptr, *scal = nullptr;
    int* bad = nullptr;
    int8_t* fixed_dof = nullptr;             // [ntotal] 1 on the dofs of fixed nodes (reactions), built on first use
    int64_t iters_total = 0, iters_last = 0;
    double res_last = 0.0;
    int64_t newton_total = 0, newton_last = 0;
    double newton_res = 0.0;

    ~svl_xnm() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
    template <class T>
    int alloc(size_t n, T** out) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
            set_error("cudaMalloc of %zu bytes failed", n * sizeof(T));
            return SVL_ERR_NOMEM;
        }
        allocs.push_back(p);
        XCUDA(cudaMemsetAsync(p, 0, std::max<size_t>(n, 1) * sizeof(T), stream));
        *out = static_cast<T*>(p);
        return SVL_OK;
    }
    template <class T>
    int upload(const std::vector<T>& h, T** out) {
        XTRY(alloc(h.size(), out));
        if (!h.empty()) XCUDA(cudaMemcpyAsync(*out, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
        return SVL_OK;
    }
};

namespace {

int grid_of(int n) { return (n + 255) / 256; }

// y_total = sum over elements of the solid / PML kernels' vectors, gathered
int x_gather(svl_xnm* X, double* y, double cn, const double* xn, double cdp, const double* xdp, int k, bool fext) {
    XGather G{};
    G.ntotal = X->m.ntotal; G.inv_ptr = X->inv_ptr; G.inv_idx = X->inv_idx; G.fe = X->fe;
    G.nodemass = X->nodemass; G.cn = cn; G.xn = xn;
    G.dp_ptr = X->dp_ptr; G.dp_col = X->dp_col; G.dp_eta = X->dp_eta; G.cdp = cdp; G.xdp = xdp;
    G.k = k; G.with_fext = fext ? 1 : 0;
    G.ld_ptr = X->ld_ptr; G.ld_ser = X->ld_ser; G.ld_coef = X->ld_coef; G.s_ptr = X->s_ptr; G.s_val = X->s_val;
    if (fext && X->ndrm > 0) { G.drm_ptr = X->drm_ptr; G.drm_idx = X->drm_idx; G.drm_fe = X->drm_fe; }
    G.y = y;
    k_xgather<<<grid_of(X->m.ntotal), 256, 0, X->stream>>>(G);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}

XSolid solid_args(svl_xnm* X) {
    XSolid S{};
    S.n = X->nsol; S.ngp = X->m.ngp; S.edof = X->s_edof; S.egeo = X->s_egeo; S.geo = X->s_geo;
    S.coef = X->s_coef; S.kind = X->s_kind; S.ctan = X->s_ctan; S.geo_f = X->s_geo_f; S.ctan_f = X->s_ctan_f;
    S.ray = X->s_ray; S.mlump = X->s_mlump; S.ftol = -1.0; S.yscale = 1.0;
    S.y = X->fe;
    return S;
}
// solid element states and filtered internal forces from X->Us
int x_state(svl_xnm* X) {
    if (X->nsol <= 0) return SVL_OK;
    XState S{};
    S.n = X->nsol; S.ngp = X->m.ngp; S.edof = X->s_edof; S.egeo = X->s_egeo; S.geo = X->s_geo;
    S.coef = X->s_coef; S.kind = X->s_kind; S.j2p = X->s_j2p; S.state = X->s_state; S.ctan = X->s_ctan;
    S.ctan_f = X->s_ctan_f;
    S.Us = X->Us; S.ftol = X->opts.ftol; S.fint = X->s_fint;
    const int g = (S.n + 127) / 128;
    if (X->m.ndim == 2) k_xstate<2, 4><<<g, 128, 0, X->stream>>>(S);
    else k_xstate<3, 8><<<g, 128, 0, X->stream>>>(S);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}
PmlArgs pml_args(svl_xnm* X) {
    PmlArgs P{};
    P.nelem = X->npml; P.X = X->p_X; P.mat = X->p_mat; P.thick = X->p_thick; P.par = X->p_par;
    P.edof = X->p_edof; P.y = X->fe + (size_t)X->nsol * X->ncs; P.ftol = -1.0; P.yscale = 1.0;
    P.tab = X->p_tab;
    return P;
}
int launch_solid(svl_xnm* X, const XSolid& S, bool single = false) {
    if (S.n <= 0) return SVL_OK;
    const int g = (S.n + 127) / 128;
    const bool one = S.xK && S.xK2 == S.xK && S.xM == S.xK && S.xM2 == S.xK && S.mlump &&
                     (!single || (S.opf && S.xK_f && S.y_f));
    if (one) {                                 // operator application: Gauss-point threads
        const int nen = X->m.nen;
        const int gg = (int)(((int64_t)S.n * nen + 127) / 128);
        if (single) {
            if (X->m.ndim == 2) k_xsolid_gp<2, 4, float><<<gg, 128, 0, X->stream>>>(S);
            else k_xsolid_gp<3, 8, float><<<gg, 128, 0, X->stream>>>(S);
        } else {
            if (X->m.ndim == 2) k_xsolid_gp<2, 4, double><<<gg, 128, 0, X->stream>>>(S);
            else k_xsolid_gp<3, 8, double><<<gg, 128, 0, X->stream>>>(S);
        }
        XCUDA(cudaGetLastError());
        return SVL_OK;
    }
    if (single) {
        if (X->m.ndim == 2) k_xsolid<2, 4, float><<<g, 128, 0, X->stream>>>(S);
        else k_xsolid<3, 8, float><<<g, 128, 0, X->stream>>>(S);
    } else {
        if (X->m.ndim == 2) k_xsolid<2, 4, double><<<g, 128, 0, X->stream>>>(S);
        else k_xsolid<3, 8, double><<<g, 128, 0, X->stream>>>(S);
    }
    XCUDA(cudaGetLastError());
    return SVL_OK;
}

// out_total = (K + 4/dt^2 M + 2/dt C + dt/3 G) p_total; single: element
// arithmetic in single precision (inner MINRES iterations)
int x_op_total(svl_xnm* X, const double* p, double* out, bool single = false, const float* p_f = nullptr) {
    const double dt = X->opts.dt, cm = 4.0 / dt / dt, cc = 2.0 / dt;
    // the single-precision data path needs the float copy of p
    if (single && !p_f) single = false;
    XSolid S = solid_args(X);
    S.xK = p; S.xK2 = p; S.cK2 = cc; S.xM = p; S.sM = cm; S.xM2 = p; S.cM2 = cc;
    S.opf = X->s_opf;                          // built for exactly these coefficients
    if (single) { S.xK_f = p_f; S.y_f = X->fe_f; }
    XTRY(launch_solid(X, S, single));
    PmlArgs P = pml_args(X);
    P.single = single ? 1 : 0;
    P.coef[0] = cm; P.coef[1] = cc; P.coef[2] = 1.0; P.coef[3] = (X->m.ndim == 3 && !X->newmark) ? dt / 3.0 : 0.0;
    for (int i = 0; i < 4; ++i) P.u[i] = p;
    if (single) { P.u_f = p_f; P.y_f = X->fe_f + (size_t)X->nsol * X->ncs; }
    XTRY(pml_action_launch(X->m.ndim, P, X->stream));
    if (!single) return x_gather(X, out, cm, p, cc, p, 0, false);
    k_xgather_f<<<grid_of(X->m.ntotal), 256, 0, X->stream>>>(X->m.ntotal, X->inv_ptr, X->inv_idx, X->fe_f, X->nodemass,
                                                             cm, p, X->dp_ptr, X->dp_col, X->dp_eta, cc, p, out);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}

// q_free = T^T Keff T v
int x_apply(svl_xnm* X, const double* v, double* q, bool single = false) {
    k_xexpand<<<grid_of(X->m.ntotal), 256, 0, X->stream>>>(X->m.ntotal, X->Tp, X->Tc, X->Tv, v, X->pt,
                                                           single ? X->pt_f : nullptr);
    XTRY(x_op_total(X, X->pt, X->yt, single, single ? X->pt_f : nullptr));
    k_xreduce<<<grid_of(X->m.nfree), 256, 0, X->stream>>>(X->m.nfree, X->TTp, X->TTr, X->TTv, X->yt, nullptr, q);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}

int x_dot(svl_xnm* X, const double* a, const double* b2, int slot) {
    k_xdot_partial<<<kBlocks, kThreads, 0, X->stream>>>(a, b2, X->m.nfree, X->partial);
    k_xdot_final<<<1, kThreads, 0, X->stream>>>(X->partial, X->scal + slot);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}
int x_read(svl_xnm* X, int slot, double* out) {
    XCUDA(cudaMemcpyAsync(out, X->scal + slot, sizeof(double), cudaMemcpyDeviceToHost, X->stream));
    XCUDA(cudaStreamSynchronize(X->stream));
    return SVL_OK;
}

// Preconditioned MINRES on T^T Keff T x = b from x = 0, restarted from its
// iterate until the true residual meets ||b - A x||_{D^-1} <= tol ||b||_{D^-1}
// with D = |diag(A)| (the norm MINRES minimises with this preconditioner; the
// plain 2-norm mixes displacement rows ~1e9 and stress rows ~1e-4 in PML models).
// The true residual always uses the double-precision operator; the inner
// iterations may apply it in single precision (opts.single_inner): FP64
// arithmetic is the scarce resource on this GPU and the element kernels are
// bound by it, while the restarts keep the result's accuracy.
int x_solve(svl_xnm* X) {
    const int n = X->m.nfree, g = grid_of(n);
    X->iters_last = 0;
    X->res_last = 0.0;
    if (n == 0) return SVL_OK;
    XCUDA(cudaMemsetAsync(X->x, 0, sizeof(double) * n, X->stream));
    k_xvmul<<<g, 256, 0, X->stream>>>(n, X->dinv, X->b, X->yv);
    XTRY(x_dot(X, X->b, X->yv, 0));
    double bs2 = 0.0;
    XTRY(x_read(X, 0, &bs2));
    if (!std::isfinite(bs2)) { set_error("non-finite effective force"); return SVL_ERR_NONFINITE; }
    if (bs2 == 0.0) return SVL_OK;
    const double bs = std::sqrt(bs2), tol = X->opts.tol;
    int64_t its = 0;
    bool done = false;
    for (int restart = 0; restart < 100 && !done; ++restart) {
        // r1 = b - A x, y = D^-1 r1, beta1 = ||r1||_{D^-1}
        if (restart == 0) {
            XCUDA(cudaMemcpyAsync(X->r1, X->b, sizeof(double) * n, cudaMemcpyDeviceToDevice, X->stream));
        } else {
            XTRY(x_apply(X, X->x, X->tmp));
            k_xsub<<<g, 256, 0, X->stream>>>(n, X->b, X->tmp, X->r1);
        }
        k_xvmul<<<g, 256, 0, X->stream>>>(n, X->dinv, X->r1, X->yv);
        XCUDA(cudaMemcpyAsync(X->r2, X->r1, sizeof(double) * n, cudaMemcpyDeviceToDevice, X->stream));
        XTRY(x_dot(X, X->r1, X->yv, 0));
        double b1 = 0.0;
        XTRY(x_read(X, 0, &b1));
        if (!std::isfinite(b1)) { set_error("MINRES: non-finite residual"); return SVL_ERR_BREAKDOWN; }
        const double beta1 = std::sqrt(b1);
        X->res_last = beta1 / bs;
        if (X->res_last <= tol) { done = true; break; }
        if (its >= X->opts.maxit) break;
        double beta = beta1, oldb = 0.0, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0;
        XCUDA(cudaMemsetAsync(X->w, 0, sizeof(double) * n, X->stream));
        XCUDA(cudaMemsetAsync(X->w2, 0, sizeof(double) * n, X->stream));
        // the recurrence estimates ||r||_{D^-1}; with single-precision inner
        // iterations each restart reduces the residual by at most 1e-5 before
        // the double-precision true residual is formed again (iterative
        // refinement: the final test is always on the double operator)
        const bool single = X->opts.single_inner != 0;
        const double inner = single ? std::max(0.5 * tol * bs, 1e-5 * beta1) : 0.5 * tol * bs;
        for (int it = 0; its < X->opts.maxit; ++it) {
            ++its;
            // v = y / beta; y = A v - (beta / oldb) r1 - (alfa / beta) r2
            k_xaxpby<<<g, 256, 0, X->stream>>>(n, 1.0 / beta, X->yv, 0.0, X->v);
            XTRY(x_apply(X, X->v, X->yv, single));
            if (it > 0) k_xaxpby<<<g, 256, 0, X->stream>>>(n, -beta / oldb, X->r1, 1.0, X->yv);
            XTRY(x_dot(X, X->v, X->yv, 1));
            double alfa = 0.0;
            XTRY(x_read(X, 1, &alfa));
            k_xaxpby<<<g, 256, 0, X->stream>>>(n, -alfa / beta, X->r2, 1.0, X->yv);
            std::swap(X->r1, X->r2);                 // r1 <- r2
            std::swap(X->r2, X->yv);                 // r2 <- y; the old r1 buffer becomes y
            k_xvmul<<<g, 256, 0, X->stream>>>(n, X->dinv, X->r2, X->yv);
            oldb = beta;
            XTRY(x_dot(X, X->r2, X->yv, 2));
            double bb = 0.0;
            XTRY(x_read(X, 2, &bb));
            if (!std::isfinite(alfa) || !std::isfinite(bb) || bb < 0.0) {
                set_error("MINRES breakdown (alpha %g, beta^2 %g)", alfa, bb);
                return SVL_ERR_BREAKDOWN;
            }
            beta = std::sqrt(bb);
            const double oldeps = epsln;
            const double delta = cs * dbar + sn * alfa;
            const double gbar = sn * dbar - cs * alfa;
            epsln = sn * beta;
            dbar = -cs * beta;
            const double gamma = std::max(std::sqrt(gbar * gbar + beta * beta), 1e-300);
            cs = gbar / gamma;
            sn = beta / gamma;
            const double phi = cs * phibar;
            phibar = sn * phibar;
            std::swap(X->w1, X->w2);                 // w1 <- w2, w2 <- w, w <- new
            std::swap(X->w2, X->w);
            k_xmr_w<<<g, 256, 0, X->stream>>>(n, X->v, X->w1, X->w2, X->w, X->x, oldeps, delta, 1.0 / gamma, phi);
            XCUDA(cudaGetLastError());
            if (phibar <= inner || beta == 0.0) break;
        }
    }
    X->iters_last = its;
    X->iters_total += its;
    if (!done) {
        set_error("MINRES did not reach %g in %lld iterations (scaled residual %g)", tol, (long long)its, X->res_last);
        return SVL_ERR_MAXITER;
    }
    return SVL_OK;
}

// ExtendedNewmarkBeta (ExtendedNewmarkBeta.cpp:208-229, 190-204):
//   b = T^T (Fext - Fint - G Wg + C V + M W) - T^T (Keff SM),
//   W = 4/dt V + A, Wg = Ubar + dt U + dt^2/6 V (set once per step);
// NewmarkBeta (NewmarkBeta.cpp:180-235):
//   b = T^T (Fext - Fint + M W + C Vd) - T^T (Keff SM),
//   W = 4/dt V + A - 4/dt^2 dU, Vd = V - 2/dt dU (set here, in Wg).
// Fint of the solid elements from their stored forces, of the PML elements
// K_e (U + T dU) (PML3DHexa8.cpp:716-742 with the node increments of the
// iterate); dUt, SM and the DRM forces of the step must be in place.
int x_rhs(svl_xnm* X, int k) {
    const HostModel& m = X->m;
    const int nt = m.ntotal, gt = grid_of(nt);
    const double dt = X->opts.dt;
    if (X->newmark) k_xrhs_nm<<<gt, 256, 0, X->stream>>>(nt, X->V, X->A, X->dUt, dt, X->W, X->Wg);
    const double* vd = X->newmark ? X->Wg : X->V;
    const size_t ns = (size_t)X->nsol * X->ncs;
    if (ns > 0) k_xneg<<<(unsigned)((ns + 255) / 256), 256, 0, X->stream>>>(ns, X->s_fint, X->fe);
    XSolid S = solid_args(X);
    S.xK2 = vd; S.cK2 = 1.0; S.xM = X->W; S.sM = 1.0; S.xM2 = vd; S.cM2 = 1.0; S.accumulate = 1;
    XTRY(launch_solid(X, S));
    if (X->npml > 0) {
        // PML: -Fint(U + T dU) filtered, then + M W + C vd (- G Wg)
        k_xadd<<<gt, 256, 0, X->stream>>>(nt, X->U, X->dUt, X->Ui);
        PmlArgs P = pml_args(X);
        P.coef[2] = 1.0; P.u[2] = X->Ui; P.ftol = X->opts.ftol; P.yscale = -1.0;
        XTRY(pml_action_launch(m.ndim, P, X->stream));
        P = pml_args(X);
        P.coef[0] = 1.0; P.u[0] = X->W; P.coef[1] = 1.0; P.u[1] = vd;
        if (m.ndim == 3 && !X->newmark) { P.coef[3] = -1.0; P.u[3] = X->Wg; }
        P.accumulate = 1;
        XTRY(pml_action_launch(m.ndim, P, X->stream));
    }
    XTRY(x_gather(X, X->yt, 1.0, X->W, 1.0, vd, k, true));
    const double* sub = nullptr;
    if (X->lt.has_sm) {
        XTRY(x_op_total(X, X->sm, X->ys));       // Keff (current tangent) SM
        sub = X->ys;
    }
    k_xreduce<<<grid_of(m.nfree), 256, 0, X->stream>>>(m.nfree, X->TTp, X->TTr, X->TTv, X->yt, sub, X->b);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}

// One ExtendedNewmarkBeta step k with the Linear algorithm (one iteration)
// or NewtonRaphson (NewtonRaphson.cpp:24-75): effective force, tangent
// solve, dU += du, convergence test (Algorithm.cpp:122-188), solid states
// from U + T dU; then the step's state update (:123-153).
int x_step(svl_xnm* X, int k) {
    const HostModel& m = X->m;
    const int nt = m.ntotal, gt = grid_of(nt), nf = m.nfree;
    const double dt = X->opts.dt;
    if (!X->newmark) k_xrhs_vec<<<gt, 256, 0, X->stream>>>(nt, X->U, X->V, X->A, X->Ub, dt, X->W, X->Wg);
    XCUDA(cudaMemsetAsync(X->dUt, 0, sizeof(double) * nt, X->stream));
    if (X->ndrm > 0) {
        XDrm D{};
        D.n = X->ndrm; D.nt = X->drm_nt; D.k = k; D.ngp = m.ngp;
        D.sidx = X->drm_sidx; D.factor = X->drm_factor; D.ak = X->drm_ak; D.node_of = X->drm_node_of;
        D.row = X->drm_row; D.ext = X->drm_ext; D.motion = X->drm_motion;
        D.egeo = X->s_egeo; D.geo = X->s_geo; D.coef = X->s_coef; D.fe = X->drm_fe;
        const int gd = (X->ndrm + 127) / 128;
        if (m.ndim == 2) k_xdrm<2, 4><<<gd, 128, 0, X->stream>>>(D);
        else k_xdrm<3, 8><<<gd, 128, 0, X->stream>>>(D);
        XCUDA(cudaGetLastError());
    }
    // the support-motion increment of step k (ExtendedNewmarkBeta.cpp:196) or
    // of step k - 1 (NewmarkBeta.cpp:187)
    if (X->lt.has_sm)
        k_xsm<<<gt, 256, 0, X->stream>>>(nt, X->sm_ptr, X->sm_ser, X->sm_fac, X->s_ptr, X->s_val,
                                         X->newmark ? k - 1 : k, X->sm);
    XCUDA(cudaMemsetAsync(X->dUf, 0, sizeof(double) * std::max(nf, 1), X->stream));
    const int maxit = X->newton ? X->opts.newton_maxit : 1;
    const int test = X->opts.cnvgtest;
    double norm0 = 0.0, res = 0.0;
    int it = 0;
    for (;;) {
        XTRY(x_rhs(X, k));
        XTRY(x_solve(X));                         // x = du; b is left as it was
        k_xaxpby<<<grid_of(nf), 256, 0, X->stream>>>(nf, 1.0, X->x, 1.0, X->dUf);
        if (X->newton) {
            // the norms the convergence test reads (Algorithm.cpp:122-188)
            double fn = 0.0, dn = 0.0, Dn = 0.0, en = 0.0;
            if (test == 1 || test == 4) { XTRY(x_dot(X, X->b, X->b, 3)); XTRY(x_read(X, 3, &fn)); }
            if (test == 2 || test == 5 || test == 7) {
                XTRY(x_dot(X, X->x, X->x, 3)); XTRY(x_read(X, 3, &dn));
                XTRY(x_dot(X, X->dUf, X->dUf, 4)); XTRY(x_read(X, 4, &Dn));
            }
            if (test == 3 || test == 6) {
                k_xvmul<<<grid_of(nf), 256, 0, X->stream>>>(nf, X->x, X->b, X->tmp);
                XTRY(x_dot(X, X->tmp, X->tmp, 3)); XTRY(x_read(X, 3, &en));
            }
            res = convergence_test(test, it, std::sqrt(fn), std::sqrt(dn), std::sqrt(Dn), std::sqrt(en), norm0);
        }
        // UpdateStatesIncrements: solid states from U + T dU
        k_xexpand<<<gt, 256, 0, X->stream>>>(nt, X->Tp, X->Tc, X->Tv, X->dUf, X->dUt);
        k_xadd<<<gt, 256, 0, X->stream>>>(nt, X->U, X->dUt, X->Us);
        XCUDA(cudaGetLastError());
        XTRY(x_state(X));
        ++it;
        if (!X->newton || !(res > X->opts.cnvgtol) || it >= maxit) break;
    }
    X->newton_last = it;
    X->newton_total += it;
    X->newton_res = res;
    k_xupdate<<<gt, 256, 0, X->stream>>>(nt, X->U, X->V, X->A, X->Ub, X->Us, X->dUt, X->lt.has_sm ? X->sm : nullptr,
                                         dt, X->newmark ? 0 : 1, X->bad);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}

// Explicit scheme tables (explicit_pml_tables, svl_host.cpp) on the device.
int cdp_setup(svl_xnm* X) {
    ExplicitPmlTables T;
    XTRY(explicit_pml_tables(X->m, X->opts.dt, X->opts.mtol, X->lt, T));
    X->cd_nsn = (int)T.sfirst.size();
    XTRY(X->upload(T.sdof, &X->cd_sdof));
    XTRY(X->upload(T.Mu, &X->cd_Mu)); XTRY(X->upload(T.Cu, &X->cd_Cu)); XTRY(X->upload(T.Ku, &X->cd_Ku));
    XTRY(X->upload(T.Gu, &X->cd_Gu));
    XTRY(X->upload(T.sfirst, &X->cd_sfirst));
    XTRY(X->upload(T.Ms, &X->cd_Ms)); XTRY(X->upload(T.Cs, &X->cd_Cs)); XTRY(X->upload(T.Ks, &X->cd_Ks));
    XTRY(X->upload(T.Gs, &X->cd_Gs)); XTRY(X->upload(T.Dinv, &X->cd_Dinv));
    XTRY(X->upload(T.kinv, &X->cd_kinv));
    XTRY(X->alloc((size_t)X->m.ntotal, &X->cd_Up)); XTRY(X->alloc((size_t)X->m.ntotal, &X->cd_Ubn));
    return SVL_OK;
}

// One explicit step k of the staggered PML scheme (see k_cdp_sin).
int cdp_step(svl_xnm* X, int k) {
    const HostModel& m = X->m;
    const int nt = m.ntotal, gt = grid_of(nt);
    const double dt = X->opts.dt;
    double *x0 = X->W, *x1 = X->Wg, *x2 = X->pt;
    // displacement rows: -(solid internal force) and -(C_uS sdot + K_uS smid + G_uS Sbar), filtered
    const size_t nsv = (size_t)X->nsol * X->ncs;
    if (nsv > 0) k_xneg<<<(unsigned)((nsv + 255) / 256), 256, 0, X->stream>>>(nsv, X->s_fint, X->fe);
    k_cdp_sin<<<gt, 256, 0, X->stream>>>(nt, X->cd_sdof, X->U, X->cd_Up, X->Ub, dt, x0, x1, x2);
    if (X->npml > 0) {
        PmlArgs P = pml_args(X);
        P.coef[1] = 1.0; P.u[1] = x0; P.coef[2] = 1.0; P.u[2] = x1;
        if (m.ndim == 3) { P.coef[3] = 1.0; P.u[3] = x2; }
        P.ftol = X->opts.ftol; P.yscale = -1.0;
        XTRY(pml_action_launch(m.ndim, P, X->stream));
    }
    XTRY(x_gather(X, X->yt, 0.0, nullptr, 0.0, nullptr, k, true));     // Fext(k) - forces
    if (X->lt.has_sm)
        k_xsm<<<gt, 256, 0, X->stream>>>(nt, X->sm_ptr, X->sm_ser, X->sm_fac, X->s_ptr, X->s_val, k, X->sm);
    const int nf = m.nfree;
    k_cdp_r<<<gt, 256, 0, X->stream>>>(nt, X->cd_sdof, X->yt, X->cd_Mu, X->cd_Cu, X->cd_Ku, X->cd_Gu, dt, X->U,
                                       X->cd_Up, X->Ub, X->ys);
    k_xreduce<<<grid_of(nf), 256, 0, X->stream>>>(nf, X->TTp, X->TTr, X->TTv, X->ys, nullptr, X->b);
    k_cdp_solve<<<grid_of(nf), 256, 0, X->stream>>>(nf, X->cd_kinv, X->b, X->x);
    k_xexpand<<<gt, 256, 0, X->stream>>>(nt, X->Tp, X->Tc, X->Tv, X->x, X->Ui);
    k_cdp_u<<<gt, 256, 0, X->stream>>>(nt, X->cd_sdof, X->Ui, X->lt.has_sm ? X->sm : nullptr, dt, X->U, X->Ub,
                                       X->dUt, X->Us, X->cd_Ubn, x0, x1, x2);
    XCUDA(cudaGetLastError());
    XTRY(x_state(X));                                                   // solid states from U + du
    // stress rows: C_Su udot + K_Su umid + G_Su ubar (unfiltered), gathered
    if (X->npml > 0) {
        PmlArgs P = pml_args(X);
        P.coef[1] = 1.0; P.u[1] = x0; P.coef[2] = 1.0; P.u[2] = x1;
        if (m.ndim == 3) { P.coef[3] = 1.0; P.u[3] = x2; }
        XTRY(pml_action_launch(m.ndim, P, X->stream));
        XTRY(x_gather(X, X->ys, 0.0, nullptr, 0.0, nullptr, 0, false));
        const int gs = (X->cd_nsn + 127) / 128;
        if (m.ndim == 2)
            k_cdp_s<3><<<gs, 128, 0, X->stream>>>(X->cd_nsn, X->cd_sfirst, X->ys, X->cd_Ms, X->cd_Cs, X->cd_Ks,
                                                  X->cd_Gs, X->cd_Dinv, X->U, X->cd_Up, X->Ub, dt, X->dUt, X->cd_Ubn);
        else
            k_cdp_s<6><<<gs, 128, 0, X->stream>>>(X->cd_nsn, X->cd_sfirst, X->ys, X->cd_Ms, X->cd_Cs, X->cd_Ks,
                                                  X->cd_Gs, X->cd_Dinv, X->U, X->cd_Up, X->Ub, dt, X->dUt, X->cd_Ubn);
    }
    k_cdp_update<<<gt, 256, 0, X->stream>>>(nt, X->U, X->cd_Up, X->V, X->A, X->Ub, X->dUt, X->cd_Ubn, dt, X->bad);
    XCUDA(cudaGetLastError());
    return SVL_OK;
}

int x_setup(svl_xnm* X, const svl_load_desc* L) {
    HostModel& m = X->m;
    const int nd = m.ndim, nen = m.nen, pnd = m.pml_ndof();
    const int npar = 3 + 2 * nd, per = nen * nd + 1;
    X->ncs = nen * nd;
    X->ncp = nen * pnd;
    std::vector<int> sol, pml;
    for (int e = 0; e < m.nelem; ++e) ((m.has_pml() && m.epml[e]) ? pml : sol).push_back(e);
    X->nsol = (int)sol.size();
    X->npml = (int)pml.size();
    // flat element-vector index of (element, local dof), element-tag order per dof
    std::vector<int64_t> base(m.nelem);
    std::vector<int> ncount(m.nelem);
    {
        int is = 0, ip = 0;
        for (int e = 0; e < m.nelem; ++e) {
            if (m.has_pml() && m.epml[e]) { base[e] = (int64_t)X->nsol * X->ncs + (int64_t)ip * X->ncp; ncount[e] = X->ncp; ++ip; }
            else { base[e] = (int64_t)is * X->ncs; ncount[e] = X->ncs; ++is; }
        }
    }
    auto gdof = [&](int e, int i) {
        const int k = ncount[e] == X->ncs ? nd : pnd;
        const int n = m.conn[(size_t)e * nen + i / k];
        return m.tdof_all[(size_t)n * m.dstride + i % k];
    };
    std::vector<int64_t> inv_ptr(m.ntotal + 1, 0), inv_idx;
    for (int e = 0; e < m.nelem; ++e)
        for (int i = 0; i < ncount[e]; ++i) inv_ptr[gdof(e, i) + 1]++;
    for (int t = 0; t < m.ntotal; ++t) inv_ptr[t + 1] += inv_ptr[t];
    inv_idx.resize(inv_ptr.back());
    {
        std::vector<int64_t> fill(inv_ptr.begin(), inv_ptr.end() - 1);
        for (int e = 0; e < m.nelem; ++e)
            for (int i = 0; i < ncount[e]; ++i) inv_idx[fill[gdof(e, i)]++] = base[e] + i;
    }
    // solid tables
    std::vector<int32_t> s_edof((size_t)X->nsol * X->ncs), s_egeo(X->nsol);
    std::vector<double> s_geo, s_coef((size_t)X->nsol * 3), s_ray, s_ml((size_t)X->nsol * nen),
        s_j2p((size_t)X->nsol * 5, 0.0);
    std::vector<int32_t> s_kind(X->nsol, 0);
    std::vector<double> diag(m.ntotal, 0.0);
    const double dt = X->opts.dt, cm = 4.0 / dt / dt, cc = 2.0 / dt;
    {
        std::map<std::vector<double>, int> seen;
        std::vector<double> buf((size_t)m.ngp * per);
        if (!m.ray.empty()) s_ray.assign((size_t)X->nsol * 2, 0.0);
        for (int i = 0; i < X->nsol; ++i) {
            const int e = sol[i];
            for (int j = 0; j < X->ncs; ++j) s_edof[(size_t)i * X->ncs + j] = gdof(e, j);
            double mab[8][8] = {};
            const double* pr = m.param(e);
            const double rho = pr[2];
            for (int q = 0; q < m.ngp; ++q) {
                double dNx[8][3], N[8];
                const double det = gp_geometry(m, e, q, dNx, N);
                for (int a = 0; a < nen; ++a)
                    for (int j = 0; j < nd; ++j) buf[(size_t)q * per + a * nd + j] = dNx[a][j];
                buf[(size_t)q * per + per - 1] = gp_factor(m, e, det);
                const double c = nd == 2 ? 1.0 * rho * m.thick[e] * std::fabs(det) : 1.0 * rho * std::fabs(det);
                for (int a = 0; a < nen; ++a)
                    for (int b2 = 0; b2 < nen; ++b2) mab[a][b2] += c * (N[a] * N[b2]);
            }
            auto it = seen.find(buf);
            if (it == seen.end()) {
                it = seen.emplace(buf, (int)(s_geo.size() / ((size_t)m.ngp * per))).first;
                s_geo.insert(s_geo.end(), buf.begin(), buf.end());
            }
            s_egeo[i] = it->second;
            // row-sum lumping in the reference's order (lin2DQuad4.cpp:272-282)
            for (int a = 0; a < nen; ++a) {
                double d = mab[a][a];
                for (int b2 = 0; b2 < nen; ++b2) if (b2 != a) d += mab[a][b2];
                s_ml[(size_t)i * nen + a] = std::fabs(d) > X->opts.mtol ? d : 0.0;
            }
            double c1, c2, c3;
            const int mt = m.mat_type(e);
            if (mt == SVL_MAT_ELASTIC2DPLANESTRAIN || mt == SVL_MAT_ELASTIC3DLINEAR) {
                const double E = pr[0], nu = pr[1];
                c1 = E * (1.0 - nu) / (1.0 - 2.0 * nu) / (1.0 + nu);
                c2 = E * nu / (1.0 - 2.0 * nu) / (1.0 + nu);
                c3 = E / (2.0 * (1.0 + nu));
            } else {
                // J2 (K, G, rho, H, beta, SY): initial tangent K 1(x)1 + 2G (I - 1/3 1(x)1)
                // with shear entries 1/2 (PlasticPlaneStrainJ2.cpp:163-180)
                const double K = pr[0], G = pr[1];
                c1 = K * 1.0 + 2.0 * G * (1.0 - 1.0 / 3.0);
                c2 = K * 1.0 + 2.0 * G * (0.0 - 1.0 / 3.0);
                c3 = 2.0 * G * 0.5;
                s_kind[i] = 1;
                s_j2p[5 * (size_t)i] = K; s_j2p[5 * (size_t)i + 1] = G; s_j2p[5 * (size_t)i + 2] = pr[3];
                s_j2p[5 * (size_t)i + 3] = pr[4]; s_j2p[5 * (size_t)i + 4] = pr[5];
                X->has_j2 = true;
            }
            s_coef[3 * i] = c1; s_coef[3 * i + 1] = c2; s_coef[3 * i + 2] = c3;
            const double am = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e], ak = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e + 1];
            if (!s_ray.empty()) { s_ray[2 * i] = am; s_ray[2 * i + 1] = ak; }
            // diagonal of the element's K + 4/dt^2 M + 2/dt C
            for (int q = 0; q < m.ngp; ++q) {
                const double* g = &buf[(size_t)q * per];
                const double w = g[per - 1];
                for (int a = 0; a < nen; ++a) {
                    const double bx = g[a * nd], by = g[a * nd + 1], bz = nd == 3 ? g[a * nd + 2] : 0.0;
                    double kd[3];
                    if (nd == 2) { kd[0] = w * (c1 * bx * bx + c3 * by * by); kd[1] = w * (c1 * by * by + c3 * bx * bx); }
                    else {
                        kd[0] = w * (c1 * bx * bx + c3 * (by * by + bz * bz));
                        kd[1] = w * (c1 * by * by + c3 * (bx * bx + bz * bz));
                        kd[2] = w * (c1 * bz * bz + c3 * (bx * bx + by * by));
                    }
                    for (int j = 0; j < nd; ++j) diag[gdof(e, a * nd + j)] += (1.0 + cc * ak) * kd[j];
                }
            }
            for (int a = 0; a < nen; ++a)
                for (int j = 0; j < nd; ++j) diag[gdof(e, a * nd + j)] += (cm + cc * am) * s_ml[(size_t)i * nen + a];
        }
    }
    // PML tables
    std::vector<double> p_X((size_t)X->npml * nen * nd), p_mat((size_t)X->npml * 3), p_thick(X->npml, 1.0),
        p_par((size_t)X->npml * npar);
    std::vector<int32_t> p_edof((size_t)X->npml * X->ncp);
    for (int i = 0; i < X->npml; ++i) {
        const int e = pml[i];
        for (int a = 0; a < nen; ++a)
            for (int j = 0; j < nd; ++j) p_X[((size_t)i * nen + a) * nd + j] = m.X[(size_t)m.conn[(size_t)e * nen + a] * nd + j];
        const double* pr = m.param(e);
        p_mat[3 * i] = pr[0]; p_mat[3 * i + 1] = pr[1]; p_mat[3 * i + 2] = pr[2];
        if (nd == 2) p_thick[i] = m.thick[e];
        for (int j = 0; j < npar; ++j) p_par[(size_t)i * npar + j] = m.pml_par[(size_t)e * npar + j];
        for (int j = 0; j < X->ncp; ++j) p_edof[(size_t)i * X->ncp + j] = gdof(e, j);
    }
    // T and T^T
    std::vector<int32_t> Tp, Tc;
    std::vector<double> Tv;
    build_total_to_free(m, Tp, Tc, Tv);
    std::vector<int32_t> TTp(m.nfree + 1, 0), TTr(Tc.size());
    std::vector<double> TTv(Tc.size());
    for (int32_t c : Tc) TTp[c + 1]++;
    for (int f = 0; f < m.nfree; ++f) TTp[f + 1] += TTp[f];
    {
        std::vector<int32_t> fill(TTp.begin(), TTp.end() - 1);
        for (int t = 0; t < m.ntotal; ++t)
            for (int i = Tp[t]; i < Tp[t + 1]; ++i) { const int p = fill[Tc[i]]++; TTr[p] = t; TTv[p] = Tv[i]; }
    }
    XTRY(build_load_tables(m, L, X->lt));
    if (L && L->ndrm > 0) {
        if (!L->drm_elem || !L->drm_factor || !L->drm_node_row || !L->drm_node_ext || !L->drm_motion || L->drm_nt <= 0) {
            set_error("domain-reduction arrays are NULL or drm_nt <= 0"); return SVL_ERR_INVALID;
        }
        std::vector<int32_t> sidx_of(m.nelem, -1);
        for (int i = 0; i < X->nsol; ++i) sidx_of[sol[i]] = i;
        std::vector<int32_t> dsidx, dnode, drow(L->drm_node_row, L->drm_node_row + m.nnode),
            dext(L->drm_node_ext, L->drm_node_ext + m.nnode), dptr(m.ntotal + 1, 0), didx;
        std::vector<double> dfac, dak;
        int nblk = 0;
        for (int r : drow) nblk = std::max(nblk, r + 1);
        std::vector<double> dmot(L->drm_motion, L->drm_motion + (size_t)nblk * L->drm_nt * 3 * nd);
        for (int i = 0; i < L->ndrm; ++i) {
            const int e = L->drm_elem[i];
            if (e < 0 || e >= m.nelem || sidx_of[e] < 0) { set_error("DRM entry %d: element %d is not a solid element", i, e); return SVL_ERR_INVALID; }
            if (s_kind[sidx_of[e]]) {
                set_error("DRM entry %d: element %d has a J2 material (the GPU DRM forces use the elastic stiffness)", i, e);
                return SVL_ERR_UNSUPPORTED;
            }
            dsidx.push_back(sidx_of[e]);
            dfac.push_back(L->drm_factor[i]);
            dak.push_back(m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e + 1]);
            for (int a = 0; a < nen; ++a) {
                const int n = m.conn[(size_t)e * nen + a];
                if (drow[n] < 0) { set_error("DRM element %d: node %d has no free-field motion", e, n); return SVL_ERR_INVALID; }
                dnode.push_back(n);
                for (int c = 0; c < nd; ++c) dptr[gdof(e, a * nd + c) + 1]++;
            }
        }
        for (int t = 0; t < m.ntotal; ++t) dptr[t + 1] += dptr[t];
        didx.resize(dptr.back());
        std::vector<int32_t> fill(dptr.begin(), dptr.end() - 1);
        for (int i = 0; i < L->ndrm; ++i)
            for (int j = 0; j < X->ncs; ++j) didx[fill[gdof(L->drm_elem[i], j)]++] = i * X->ncs + j;
        X->ndrm = L->ndrm;
        X->drm_nt = L->drm_nt;
        XTRY(X->upload(dsidx, &X->drm_sidx)); XTRY(X->upload(dfac, &X->drm_factor)); XTRY(X->upload(dak, &X->drm_ak));
        XTRY(X->upload(dnode, &X->drm_node_of)); XTRY(X->upload(drow, &X->drm_row)); XTRY(X->upload(dext, &X->drm_ext));
        XTRY(X->upload(dmot, &X->drm_motion)); XTRY(X->upload(dptr, &X->drm_ptr)); XTRY(X->upload(didx, &X->drm_idx));
        XTRY(X->alloc((size_t)X->ndrm * X->ncs, &X->drm_fe));
    }
    // uploads
    XTRY(X->upload(s_edof, &X->s_edof)); XTRY(X->upload(s_egeo, &X->s_egeo)); XTRY(X->upload(s_geo, &X->s_geo));
    {
        std::vector<float> gf(s_geo.begin(), s_geo.end());
        XTRY(X->upload(gf, &X->s_geo_f));
        // single-precision operator constants of Keff = K + 4/dt^2 M + 2/dt C
        std::vector<float> opf((size_t)X->nsol * (nen + 4));
        for (int i = 0; i < X->nsol; ++i) {
            const int e = sol[i];
            const double am = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e], ak = m.ray.empty() ? 0.0 : m.ray[2 * (size_t)e + 1];
            float* o = &opf[(size_t)i * (nen + 4)];
            for (int a = 0; a < nen; ++a) o[a] = (float)(s_ml[(size_t)i * nen + a] * (cm + cc * am));
            o[nen] = (float)(cc * ak);
            for (int j = 0; j < 3; ++j) o[nen + 1 + j] = (float)s_coef[3 * (size_t)i + j];
        }
        XTRY(X->upload(opf, &X->s_opf));
    }
    XTRY(X->upload(s_coef, &X->s_coef)); XTRY(X->upload(s_ml, &X->s_mlump));
    XTRY(X->alloc((size_t)X->nsol * X->ncs, &X->s_fint));
    if (X->has_j2) {
        const int ns = nd == 2 ? 3 : 6;
        XTRY(X->upload(s_kind, &X->s_kind)); XTRY(X->upload(s_j2p, &X->s_j2p));
        XTRY(X->alloc((size_t)kJ2State * m.ngp * X->nsol, &X->s_state));
        XTRY(X->alloc((size_t)ns * ns * m.ngp * X->nsol, &X->s_ctan));
        XTRY(X->alloc((size_t)ns * ns * m.ngp * X->nsol, &X->s_ctan_f));
    }
    if (!s_ray.empty()) XTRY(X->upload(s_ray, &X->s_ray));
    XTRY(X->upload(p_X, &X->p_X)); XTRY(X->upload(p_mat, &X->p_mat)); XTRY(X->upload(p_thick, &X->p_thick));
    XTRY(X->upload(p_par, &X->p_par)); XTRY(X->upload(p_edof, &X->p_edof));
    if (X->npml > 0) {
        std::vector<float> tab;
        pml_tab_fill(nd, X->npml, p_X.data(), p_mat.data(), nd == 2 ? p_thick.data() : nullptr, p_par.data(), tab);
        XTRY(X->upload(tab, &X->p_tab));
    }
    XTRY(X->alloc((size_t)X->nsol * X->ncs + (size_t)X->npml * X->ncp, &X->fe));
    if (X->opts.single_inner) {
        XTRY(X->alloc((size_t)X->nsol * X->ncs + (size_t)X->npml * X->ncp, &X->fe_f));
        XTRY(X->alloc((size_t)m.ntotal, &X->pt_f));
    }
    XTRY(X->upload(inv_ptr, &X->inv_ptr)); XTRY(X->upload(inv_idx, &X->inv_idx));
    if (!m.dp_eta.empty()) {                 // ZeroLength1D dashpots
        std::vector<int32_t> dpp, dpc;
        std::vector<double> dpe;
        dashpot_tables(m, dpp, dpc, dpe);
        for (size_t i = 0; i < m.dp_eta.size(); ++i) {
            diag[m.dp_dof[2 * i]] += cc * m.dp_eta[i];
            diag[m.dp_dof[2 * i + 1]] += cc * m.dp_eta[i];
        }
        XTRY(X->upload(dpp, &X->dp_ptr)); XTRY(X->upload(dpc, &X->dp_col)); XTRY(X->upload(dpe, &X->dp_eta));
    }
    if (!m.nodemass.empty()) {
        std::vector<double> nm(m.ntotal, 0.0);
        for (int t = 0; t < m.ntotal; ++t) if (std::fabs(m.nodemass[t]) > X->opts.mtol) nm[t] = m.nodemass[t];
        for (int t = 0; t < m.ntotal; ++t) diag[t] += cm * nm[t];
        XTRY(X->upload(nm, &X->nodemass));
    }
    XTRY(X->upload(Tp, &X->Tp)); XTRY(X->upload(Tc, &X->Tc)); XTRY(X->upload(Tv, &X->Tv));
    XTRY(X->upload(TTp, &X->TTp)); XTRY(X->upload(TTr, &X->TTr)); XTRY(X->upload(TTv, &X->TTv));
    XTRY(X->upload(X->lt.ld_ptr, &X->ld_ptr)); XTRY(X->upload(X->lt.ld_ser, &X->ld_ser)); XTRY(X->upload(X->lt.ld_coef, &X->ld_coef));
    XTRY(X->upload(X->lt.s_ptr, &X->s_ptr)); XTRY(X->upload(X->lt.s_val, &X->s_val));
    XTRY(X->upload(X->lt.sm_ptr, &X->sm_ptr)); XTRY(X->upload(X->lt.sm_ser, &X->sm_ser)); XTRY(X->upload(X->lt.sm_fac, &X->sm_fac));
    double** tvec[] = {&X->U, &X->V, &X->A, &X->Ub, &X->Us, &X->W, &X->Wg, &X->yt, &X->ys, &X->pt, &X->sm, &X->dUt,
                       &X->Ui};
    for (double** p : tvec) XTRY(X->alloc((size_t)m.ntotal, p));
    double** fvec[] = {&X->b, &X->x, &X->dUf, &X->r1, &X->r2, &X->yv, &X->v, &X->w, &X->w1, &X->w2, &X->tmp};
    for (double** p : fvec) XTRY(X->alloc((size_t)std::max(m.nfree, 1), p));
    XTRY(X->alloc(kBlocks, &X->partial));
    XTRY(X->alloc(8, &X->scal));
    XTRY(X->alloc(1, &X->bad));
    // PML diagonal entries by unit probes of the element action (once; the
    // explicit scheme has no solve)
    if (X->npml > 0 && !X->explicit_cd) {
        double *ub = nullptr, *yb = nullptr, *db = nullptr;
        const size_t ne = (size_t)X->npml * X->ncp;
        XTRY(X->alloc(ne, &ub)); XTRY(X->alloc(ne, &yb)); XTRY(X->alloc(ne, &db));
        PmlArgs P{};
        P.nelem = X->npml; P.X = X->p_X; P.mat = X->p_mat; P.thick = X->p_thick; P.par = X->p_par;
        P.edof = nullptr; P.y = yb; P.ftol = -1.0; P.yscale = 1.0;
        P.coef[0] = cm; P.coef[1] = cc; P.coef[2] = 1.0; P.coef[3] = (nd == 3 && !X->newmark) ? dt / 3.0 : 0.0;
        for (int i = 0; i < 4; ++i) P.u[i] = ub;
        const int gu = (int)((ne + 255) / 256), ge = grid_of(X->npml);
        for (int i = 0; i < X->ncp; ++i) {
            k_xunit<<<gu, 256, 0, X->stream>>>(X->npml, X->ncp, i, ub);
            XTRY(pml_action_launch(nd, P, X->stream));
            k_xtake<<<ge, 256, 0, X->stream>>>(X->npml, X->ncp, i, yb, db);
        }
        XCUDA(cudaGetLastError());
        std::vector<double> dh(ne);
        XCUDA(cudaMemcpyAsync(dh.data(), db, ne * sizeof(double), cudaMemcpyDeviceToHost, X->stream));
        XCUDA(cudaStreamSynchronize(X->stream));
        for (int i = 0; i < X->npml; ++i)
            for (int j = 0; j < X->ncp; ++j) diag[p_edof[(size_t)i * X->ncp + j]] += dh[(size_t)i * X->ncp + j];
    }
    if (X->explicit_cd) XTRY(cdp_setup(X));
    // Jacobi on the free dofs: |sum_t T_tf^2 diag_t|^-1
    std::vector<double> dfree(std::max(m.nfree, 1), 0.0);
    for (int t = 0; t < m.ntotal; ++t)
        for (int i = Tp[t]; i < Tp[t + 1]; ++i) dfree[Tc[i]] += Tv[i] * Tv[i] * diag[t];
    for (double& d : dfree) d = std::fabs(d) > 0.0 ? 1.0 / std::fabs(d) : 1.0;
    XTRY(X->upload(dfree, &X->dinv));
    XTRY(x_state(X));                         // Us = 0: zero forces, initial tangents
    XCUDA(cudaStreamSynchronize(X->stream));
    return SVL_OK;
}

}  // namespace

extern "C" {

int svl_xnm_create(const svl_model_desc* model, const svl_load_desc* loads, const svl_xnm_opts* opts, svl_xnm** out) {
    if (!out || !opts) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    *out = nullptr;
    const bool expl = opts->integrator == SVL_XNM_CENTRAL_DIFFERENCE;
    if (!(opts->dt > 0.0) || (!expl && (!(opts->tol > 0.0) || opts->maxit <= 0))) { set_error("bad ExtendedNewmark options"); return SVL_ERR_INVALID; }
    if (opts->algorithm != SVL_ALGO_LINEAR && opts->algorithm != SVL_ALGO_NEWTON) { set_error("unknown algorithm %d", opts->algorithm); return SVL_ERR_INVALID; }
    if (opts->algorithm == SVL_ALGO_NEWTON &&
        (opts->newton_maxit <= 0 || opts->cnvgtest < 1 || opts->cnvgtest > 8 || !(opts->cnvgtol >= 0.0))) {
        set_error("Newton needs newton_maxit > 0, cnvgtest 1..8 and cnvgtol >= 0"); return SVL_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error("no CUDA device available"); return SVL_ERR_NODEVICE; }
    svl_xnm* X = new svl_xnm();
    X->opts = *opts;
    auto fail = [&](int st) { delete X; return st; };
    if (!model_from_desc(model, X->m)) return fail(SVL_ERR_INVALID);
    X->newton = opts->algorithm == SVL_ALGO_NEWTON;
    if (opts->integrator != SVL_XNM_EXTENDED_NEWMARK && opts->integrator != SVL_XNM_NEWMARK && !expl) {
        set_error("unknown integrator %d", opts->integrator); return fail(SVL_ERR_INVALID);
    }
    X->newmark = opts->integrator == SVL_XNM_NEWMARK;
    X->explicit_cd = expl;
    if (expl) {
        const HostModel& m = X->m;
        if (opts->algorithm != SVL_ALGO_LINEAR) { set_error("the explicit PML scheme takes the Linear algorithm"); return fail(SVL_ERR_UNSUPPORTED); }
        if (!m.dp_eta.empty()) { set_error("the explicit PML scheme does not take dashpots"); return fail(SVL_ERR_UNSUPPORTED); }
        if (loads && loads->ndrm > 0) { set_error("the explicit PML scheme does not take domain-reduction loads"); return fail(SVL_ERR_UNSUPPORTED); }
        for (int e = 0; !m.ray.empty() && e < m.nelem; ++e)
            if (m.ray[2 * (size_t)e + 1] != 0.0 || (m.has_pml() && m.epml[e] && m.ray[2 * (size_t)e] != 0.0)) {
                set_error("the explicit PML scheme takes mass-proportional Rayleigh damping on solid elements only");
                return fail(SVL_ERR_UNSUPPORTED);
            }
    }
    for (int e = 0; X->m.has_pml() && e < X->m.nelem; ++e) {
        const int t = X->m.mat_type(e);
        if (X->m.epml[e] && t != SVL_MAT_ELASTIC2DPLANESTRAIN && t != SVL_MAT_ELASTIC3DLINEAR) {
            set_error("PML element %d needs an elastic material", e); return fail(SVL_ERR_INVALID);
        }
    }
    if (!X->m.lumped) { set_error("the ExtendedNewmark path needs a lumped mass for the solid elements"); return fail(SVL_ERR_UNSUPPORTED); }
    if ((int64_t)X->m.nelem * X->m.nen * X->m.pml_ndof() > ((int64_t)1 << 40)) { set_error("model too large"); return fail(SVL_ERR_UNSUPPORTED); }
    if (cudaStreamCreateWithFlags(&X->stream, cudaStreamNonBlocking) != cudaSuccess) { set_error("cudaStreamCreate failed"); return fail(SVL_ERR_CUDA); }
    int st = x_setup(X, loads);
    if (st) return fail(st);
    *out = X;
    return SVL_OK;
}

int svl_xnm_set_initial(svl_xnm* X, const double* U0, const double* V0, const double* A0, const double* Ubar0) {
    if (!X) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    const size_t bytes = sizeof(double) * X->m.ntotal;
    const double* src[4] = {U0, V0, A0, Ubar0};
    double* dst[4] = {X->U, X->V, X->A, X->Ub};
    for (int i = 0; i < 4; ++i) {
        if (src[i]) XCUDA(cudaMemcpyAsync(dst[i], src[i], bytes, cudaMemcpyHostToDevice, X->stream));
        else XCUDA(cudaMemsetAsync(dst[i], 0, bytes, X->stream));
    }
    XCUDA(cudaMemcpyAsync(X->Us, X->U, bytes, cudaMemcpyDeviceToDevice, X->stream));
    if (X->explicit_cd) {
        k_cdp_init<<<grid_of(X->m.ntotal), 256, 0, X->stream>>>(X->m.ntotal, X->U, X->V, X->A, X->opts.dt, X->cd_Up);
        XCUDA(cudaGetLastError());
    }
    XTRY(x_state(X));                         // element states from U0 (oracle: UpdateState + commit)
    XCUDA(cudaStreamSynchronize(X->stream));
    return SVL_OK;
}

int svl_xnm_run(svl_xnm* X, int32_t k_first, int32_t nsteps, double* U_hist) {
    if (!X || nsteps < 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    const size_t nt = X->m.ntotal;
    for (int i = 0; i < nsteps; ++i) {
        XTRY(X->explicit_cd ? cdp_step(X, k_first + i) : x_step(X, k_first + i));
        if (U_hist) XCUDA(cudaMemcpyAsync(U_hist + (size_t)i * nt, X->U, sizeof(double) * nt, cudaMemcpyDeviceToHost, X->stream));
    }
    int bad = 0;
    XCUDA(cudaMemcpyAsync(&bad, X->bad, sizeof(int), cudaMemcpyDeviceToHost, X->stream));
    XCUDA(cudaStreamSynchronize(X->stream));
    if (bad) { set_error("non-finite displacement"); return SVL_ERR_NONFINITE; }
    return SVL_OK;
}

int svl_xnm_get(svl_xnm* X, int32_t which, double* out) {
    if (!X || !out || which < 0 || which > 3) { set_error("bad argument"); return SVL_ERR_INVALID; }
    const double* src[4] = {X->U, X->V, X->A, X->Ub};
    XCUDA(cudaMemcpyAsync(out, src[which], sizeof(double) * X->m.ntotal, cudaMemcpyDeviceToHost, X->stream));
    XCUDA(cudaStreamSynchronize(X->stream));
    return SVL_OK;
}

// Reaction forces after step k (the step just run), as DynamicAnalysis::
// UpdateDomain stores them (DynamicAnalysis.cpp:128-150) through
// ExtendedNewmarkBeta / NewmarkBeta::ComputeReactionForce
// (ExtendedNewmarkBeta.cpp:158-172, NewmarkBeta.cpp:148-162): the dynamic
// internal force (node inertia m A; solids Fint_e + C_e V_e + M_e A_e; PML
// elements K_e u_e + C_e v_e + M_e a_e, PML3DHexa8.cpp:746-767, without the
// history term; dashpots) minus Fext(k), on the dofs of fixed nodes.  Every
// element touching such a dof has that fixed node, so all elements are
// evaluated and the other rows dropped: the element order of each row's sum
// is the reference's.  The element vectors are formed negated and the ordered
// gather adds Fext(k), so R = -(gathered vector) on those dofs.
int svl_xnm_reaction(svl_xnm* X, int32_t k, double* R) {
    if (!X || !R) { set_error("NULL argument"); return SVL_ERR_INVALID; }
    if (X->explicit_cd) {
        set_error("reaction forces are not covered for the explicit PML scheme (its stress dofs live at the half steps)");
        return SVL_ERR_UNSUPPORTED;
    }
    const HostModel& m = X->m;
    const int nt = m.ntotal, gt = grid_of(nt);
    if (!X->fixed_dof) {
        std::vector<int8_t> fx(nt, 0);
        for (int n = 0; n < m.nnode; ++n) {
            bool f = false;
            for (int j = 0; j < m.nndof[n]; ++j) f = f || m.fdof_all[(size_t)n * m.dstride + j] == -1;
            if (f)
                for (int j = 0; j < m.nndof[n]; ++j) fx[m.tdof_all[(size_t)n * m.dstride + j]] = 1;
        }
        XTRY(X->alloc(nt, &X->fixed_dof));
        XCUDA(cudaMemcpyAsync(X->fixed_dof, fx.data(), nt, cudaMemcpyHostToDevice, X->stream));
    }
    const size_t ns = (size_t)X->nsol * X->ncs;
    if (ns > 0) k_xneg<<<(unsigned)((ns + 255) / 256), 256, 0, X->stream>>>(ns, X->s_fint, X->fe);
    XSolid S = solid_args(X);
    S.xK2 = X->V; S.cK2 = -1.0; S.xM = X->A; S.sM = -1.0; S.xM2 = X->V; S.cM2 = -1.0; S.accumulate = 1;
    XTRY(launch_solid(X, S));
    if (X->npml > 0) {
        PmlArgs P = pml_args(X);
        P.coef[0] = 1.0; P.u[0] = X->A; P.coef[1] = 1.0; P.u[1] = X->V; P.coef[2] = 1.0; P.u[2] = X->U;
        P.yscale = -1.0;
        XTRY(pml_action_launch(m.ndim, P, X->stream));
    }
    XTRY(x_gather(X, X->yt, -1.0, X->A, -1.0, X->V, k, true));
    k_xreact<<<gt, 256, 0, X->stream>>>(nt, X->fixed_dof, X->yt, X->ys);
    XCUDA(cudaGetLastError());
    XCUDA(cudaMemcpyAsync(R, X->ys, sizeof(double) * nt, cudaMemcpyDeviceToHost, X->stream));
    XCUDA(cudaStreamSynchronize(X->stream));
    return SVL_OK;
}

int svl_xnm_stats(svl_xnm* X, int64_t* iters_total, int64_t* iters_last, double* res_last) {
    if (!X) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (iters_total) *iters_total = X->iters_total;
    if (iters_last) *iters_last = X->iters_last;
    if (res_last) *res_last = X->res_last;
    return SVL_OK;
}

int svl_xnm_newton_stats(svl_xnm* X, int64_t* iters_total, int64_t* iters_last, double* residual_last) {
    if (!X) { set_error("NULL handle"); return SVL_ERR_INVALID; }
    if (iters_total) *iters_total = X->newton_total;
    if (iters_last) *iters_last = X->newton_last;
    if (residual_last) *residual_last = X->newton_res;
    return SVL_OK;
}

void svl_xnm_destroy(svl_xnm* X) { delete X; }

}  // extern "C"
