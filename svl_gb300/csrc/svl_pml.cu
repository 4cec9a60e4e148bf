// PML2DQuad4 / PML3DHexa8 element action on the GPU.
//
// The reference builds the element's mass, damping, stiffness and history
// matrices (PML2DQuad4.cpp:233-494, PML3DHexa8.cpp:214-742) and multiplies
// them with nodal vectors (ComputeInternalForces = K u).  Here every thread
// applies  y_e = c_M M u_M + c_C C u_C + c_K K u_K + c_G G u_G  to one
// element without forming the 20x20 / 72x72 matrices: at each Gauss point
// the interpolated displacement U = sum N_a u_a, stress S = sum N_a s_a and
// displacement gradient grad u = sum u_a (x) dN_a are formed once and the
// three blocks of each matrix are applied through them:
//   displacement rows   rho s N_j U + q_d dN_j,d S(coupled component)
//   stress rows         N_j (compliance(s) S + q_d du/dx_d)
// with s and q the stretching combinations of each matrix (M: s = ax ay az,
// no coupling; C: s = ax ay bz + ax by az + bx ay az, q = (ay az, ax az, ax ay);
// K: s = ax by bz + bx by az + bx ay bz, q = (ay bz + az by, ax bz + az bx,
// ax by + ay bx); G: s = bx by bz, q = (by bz, bx bz, bx by); in 2D M: ax ay,
// C: ax by + ay bx with q = (ay, ax), K: bx by with q = (by, bx), no G).
#include <cmath>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "svl_internal.hpp"

using namespace svl;

namespace {

#define PML_TRY(x)                                                                   \
    do {                                                                             \
        cudaError_t err_ = (x);                                                      \
        if (err_ != cudaSuccess) {                                                   \
            set_error("%s failed: %s (%s:%d)", #x, cudaGetErrorString(err_), __FILE__, __LINE__); \
            return SVL_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)

}  // namespace

namespace svl {

// T = double: the reference's arithmetic.  T = float: the same operator in
// single precision (coordinates taken relative to the element's first node,
// material and stretching constants formed in double), for the inner
// iterations of a solve whose residual is checked with the double operator.
template <int ND, typename T>
__global__ void __launch_bounds__(128) k_pml_action(PmlArgs A) {
    constexpr int NEN = ND == 2 ? 4 : 8, NN = ND == 2 ? 5 : 9, NC = NEN * NN, NS = ND == 2 ? 3 : 6;
    constexpr int NPAR = 3 + 2 * ND;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.nelem) return;
    const double* Xd = A.X + (size_t)e * NEN * ND;
    const double E_ = A.mat[3 * e], nu_ = A.mat[3 * e + 1], rho_ = A.mat[3 * e + 2];
    const double* par = A.par + (size_t)e * NPAR;
    const double mu_ = E_ / 2.0 / (1 + nu_);
    const double lambda_ = E_ * nu_ / (1.0 + nu_) / (1.0 - 2.0 * nu_);
    const double Vp_ = sqrt((lambda_ + 2.0 * mu_) / rho_);
    const double pm_ = par[0], L_ = par[1], R_ = par[2];
    const T mu = (T)mu_, lambda = (T)lambda_, rho = (T)rho_;
    const T t = (T)((ND == 2 && A.thick) ? A.thick[e] : 1.0);
    const T pm = (T)pm_, L = (T)L_;
    const T a0 = (T)((pm_ + 1.0) * (L_ / 10.0) / 2.0 / L_ * log(1.0 / R_));
    const T b0 = (T)((pm_ + 1.0) * Vp_ / 2.0 / L_ * log(1.0 / R_));
    const T g = (T)0.577350269189626;       // GaussQuadrature.cpp:303-316
    T X[NEN * ND], xoff[3] = {0, 0, 0};       // node coordinates relative to node 0; node 0 - x0
#pragma unroll
    for (int i = 0; i < NEN * ND; ++i) X[i] = (T)(Xd[i] - Xd[i % ND]);
#pragma unroll
    for (int i = 0; i < ND; ++i) xoff[i] = (T)(Xd[i] - par[3 + i]);
    T y[NC];
#pragma unroll
    for (int i = 0; i < NC; ++i) y[i] = 0;
    // all active matrices on one input vector: a single weighted pass
    bool fused = true;
    {
        const double* u0 = nullptr;
        for (int k = 0; k < 4; ++k) {
            if (A.coef[k] == T(0.0) || (ND == 2 && k == 3)) continue;
            if (!u0) u0 = A.u[k];
            else if (A.u[k] != u0) fused = false;
        }
    }
    for (int q = 0; q < NEN; ++q) {
        const T xi[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, (q & 4) ? g : -g};
        T N[NEN], dN[NEN][3];
        if (ND == 2) {
            const T sr[4] = {-1, 1, 1, -1}, ss[4] = {-1, -1, 1, 1};
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                N[a] = T(0.25) * (T(1.0) + sr[a] * xi[0]) * (T(1.0) + ss[a] * xi[1]);
                dN[a][0] = T(0.25) * sr[a] * (T(1.0) + ss[a] * xi[1]);
                dN[a][1] = T(0.25) * ss[a] * (T(1.0) + sr[a] * xi[0]);
                dN[a][2] = T(0.0);
            }
        } else {
            const T sr[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, ss[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
            const T st[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                const T fr = T(1.0) + sr[a] * xi[0], fs = T(1.0) + ss[a] * xi[1], ft = T(1.0) + st[a] * xi[2];
                N[a] = T(0.125) * fr * fs * ft;
                dN[a][0] = T(0.125) * sr[a] * fs * ft;
                dN[a][1] = T(0.125) * ss[a] * fr * ft;
                dN[a][2] = T(0.125) * st[a] * fr * fs;
            }
        }
        T J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, xg[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int i = 0; i < ND; ++i) {
                xg[i] += N[a] * X[a * ND + i];
#pragma unroll
                for (int j = 0; j < ND; ++j) J[i][j] += dN[a][i] * X[a * ND + j];
            }
        T det, Ji[3][3];
        if (ND == 2) {
            det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
            Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
            Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
        } else {
            const T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
            det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
            Ji[0][0] = c00 / det;
            Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
            Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
            Ji[1][0] = c01 / det;
            Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
            Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
            Ji[2][0] = c02 / det;
            Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
            Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        }
        T dx[NEN][3];
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                T v = T(0.0);
                if (j < ND)
#pragma unroll
                    for (int i = 0; i < ND; ++i) v += Ji[j][i] * dN[a][i];
                dx[a][j] = v;
            }
        const T f = ND == 2 ? t * T(1.0) * fabs(det) : T(1.0) * fabs(det);
        T as[3] = {1, 1, 1}, bs[3] = {0, 0, 0};
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            const T r = pow((xoff[i] + xg[i]) * (T)par[3 + ND + i] / L, pm);
            as[i] = T(1.0) + a0 * r;
            bs[i] = b0 * r;
        }
        // stretching combinations of matrix mi (see the header)
        auto combo = [&](int mi, T& s, T& qx, T& qy, T& qz) {
            qz = T(0.0);
            if (ND == 2) {
                if (mi == 0) { s = as[0] * as[1]; qx = 0; qy = 0; }
                else if (mi == 1) { s = as[0] * bs[1] + as[1] * bs[0]; qx = as[1]; qy = as[0]; }
                else { s = bs[0] * bs[1]; qx = bs[1]; qy = bs[0]; }
            } else {
                if (mi == 0) { s = as[0] * as[1] * as[2]; qx = qy = qz = T(0.0); }
                else if (mi == 1) {
                    s = as[0] * as[1] * bs[2] + as[0] * bs[1] * as[2] + bs[0] * as[1] * as[2];
                    qx = as[1] * as[2]; qy = as[0] * as[2]; qz = as[0] * as[1];
                } else if (mi == 2) {
                    s = as[0] * bs[1] * bs[2] + bs[0] * bs[1] * as[2] + bs[0] * as[1] * bs[2];
                    qx = as[1] * bs[2] + as[2] * bs[1]; qy = as[0] * bs[2] + as[2] * bs[0]; qz = as[0] * bs[1] + as[1] * bs[0];
                } else {
                    s = bs[0] * bs[1] * bs[2];
                    qx = bs[1] * bs[2]; qy = bs[0] * bs[2]; qz = bs[0] * bs[1];
                }
            }
        };
        // Every matrix is linear in (s, q) for a fixed input vector, so when all
        // active matrices act on the same vector (an operator application) one
        // pass with the coefficient-weighted combination replaces four.
        const int npass = fused ? 1 : 4;
        for (int mi = 0; mi < npass; ++mi) {
            T c, s, qx, qy, qz;
            const double* ubase;
            if (fused) {
                c = T(1.0); s = qx = qy = qz = T(0.0);
                ubase = nullptr;
                for (int k = 0; k < 4; ++k) {
                    if (A.coef[k] == T(0.0) || (ND == 2 && k == 3)) continue;
                    T sk, xk, yk, zk;
                    combo(k, sk, xk, yk, zk);
                    const T ck = (T)A.coef[k];
                    s += ck * sk; qx += ck * xk; qy += ck * yk; qz += ck * zk;
                    ubase = A.u[k];
                }
                if (!ubase) continue;
            } else {
                c = (T)A.coef[mi];
                if (c == T(0.0) || (ND == 2 && mi == 3)) continue;
                combo(mi, s, qx, qy, qz);
                ubase = A.u[mi];
            }
            const double* u = ubase + (A.edof ? 0 : (size_t)e * NC);
            const int32_t* ed = A.edof ? A.edof + (size_t)e * NC : nullptr;
            // interpolated displacement, stress and displacement gradient
            T U[3] = {0, 0, 0}, S[NS], Gd[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int i = 0; i < NS; ++i) S[i] = T(0.0);
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const T ua = (T)(ed ? u[ed[a * NN + d]] : u[a * NN + d]);
                    U[d] += N[a] * ua;
#pragma unroll
                    for (int j = 0; j < ND; ++j) Gd[d][j] += ua * dx[a][j];
                }
#pragma unroll
                for (int i = 0; i < NS; ++i) S[i] += N[a] * (T)(ed ? u[ed[a * NN + ND + i]] : u[a * NN + ND + i]);
            }
            const T cf = c * f;
#pragma unroll
            for (int j = 0; j < NEN; ++j) {
                const T Nj = N[j];
                T* yj = y + j * NN;
                if (ND == 2) {
                    // dofs: ux uy s11 s22 s12
                    const T k2 = s * (lambda + T(2.0) * mu) / T(4.0) / mu / (lambda + mu);
                    const T l2 = s * lambda / T(4.0) / mu / (lambda + mu);
                    yj[0] += cf * (rho * s * Nj * U[0] + qx * dx[j][0] * S[0] + qy * dx[j][1] * S[2]);
                    yj[1] += cf * (rho * s * Nj * U[1] + qy * dx[j][1] * S[1] + qx * dx[j][0] * S[2]);
                    yj[2] += cf * Nj * (-k2 * S[0] + l2 * S[1] + qx * Gd[0][0]);
                    yj[3] += cf * Nj * (-k2 * S[1] + l2 * S[0] + qy * Gd[1][1]);
                    yj[4] += cf * Nj * (-s / mu * S[2] + qy * Gd[0][1] + qx * Gd[1][0]);
                } else {
                    // dofs: ux uy uz s11 s22 s33 s12 s23 s13
                    const T kap = s * (lambda + mu) / mu / (T(3.0) * lambda + T(2.0) * mu);
                    const T lam = s * lambda / T(2.0) / mu / (T(3.0) * lambda + T(2.0) * mu);
                    const T dxj = dx[j][0], dyj = dx[j][1], dzj = dx[j][2];
                    yj[0] += cf * (rho * s * Nj * U[0] + qx * dxj * S[0] + qy * dyj * S[3] + qz * dzj * S[5]);
                    yj[1] += cf * (rho * s * Nj * U[1] + qy * dyj * S[1] + qx * dxj * S[3] + qz * dzj * S[4]);
                    yj[2] += cf * (rho * s * Nj * U[2] + qz * dzj * S[2] + qx * dxj * S[5] + qy * dyj * S[4]);
                    yj[3] += cf * Nj * (-kap * S[0] + lam * (S[1] + S[2]) + qx * Gd[0][0]);
                    yj[4] += cf * Nj * (-kap * S[1] + lam * (S[0] + S[2]) + qy * Gd[1][1]);
                    yj[5] += cf * Nj * (-kap * S[2] + lam * (S[0] + S[1]) + qz * Gd[2][2]);
                    yj[6] += cf * Nj * (-s / mu * S[3] + qy * Gd[0][1] + qx * Gd[1][0]);
                    yj[7] += cf * Nj * (-s / mu * S[4] + qz * Gd[1][2] + qy * Gd[2][1]);
                    yj[8] += cf * Nj * (-s / mu * S[5] + qz * Gd[0][2] + qx * Gd[2][0]);
                }
            }
        }
    }
    double* out = A.y + (size_t)e * NC;
#pragma unroll
    for (int i = 0; i < NC; ++i) {
        double v = (double)y[i];
        if (A.ftol >= 0.0 && !(fabs(v) > A.ftol)) v = 0.0;
        v *= A.yscale;
        out[i] = A.accumulate ? out[i] + v : v;
    }
}

// The operator form of k_pml_action (every active matrix on one vector, one
// weighted pass) with one thread per (element, Gauss point): the NEN threads
// of an element are consecutive lanes, lane q loads node q's dofs and forms
// Gauss point q, node values reach the other lanes by shuffles, and a
// butterfly over the NEN lanes sums the element vector; lane q writes node q.
template <int ND, typename T>
__global__ void __launch_bounds__(128) k_pml_action_gp(PmlArgs A) {
    constexpr int NEN = ND == 2 ? 4 : 8, NN = ND == 2 ? 5 : 9, NC = NEN * NN, NS = ND == 2 ? 3 : 6;
    constexpr int NPAR = 3 + 2 * ND;
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int e = gtid / NEN, q = gtid % NEN;
    const bool valid = e < A.nelem;
    const int ec = valid ? e : A.nelem - 1;
    const int lane = threadIdx.x & 31, base = lane - q;
    T X[NEN * ND], xoff[3] = {0, 0, 0}, nrm[3] = {0, 0, 0};
    T mu, lambda, rho, a0, b0, pm, L, t;
    if constexpr (std::is_same<T, float>::value) {
        // precomputed single-precision constants (conversions from double run
        // at the FP64 rate on this GPU)
        constexpr int TS = (NEN * ND + 2 * ND + 8 + 3) / 4 * 4;      // pml_tab_stride(ND)
        const float* tb = A.tab + (size_t)ec * TS;
#pragma unroll
        for (int i = 0; i < NEN * ND; ++i) X[i] = tb[i];
#pragma unroll
        for (int i = 0; i < ND; ++i) { xoff[i] = tb[NEN * ND + i]; nrm[i] = tb[NEN * ND + ND + i]; }
        const float* c = tb + NEN * ND + 2 * ND;
        mu = c[0]; lambda = c[1]; rho = c[2]; a0 = c[3]; b0 = c[4]; pm = c[5]; L = c[6]; t = c[7];
    } else {
        const double* Xd = A.X + (size_t)ec * NEN * ND;
        const double* par = A.par + (size_t)ec * NPAR;
        const T E = (T)A.mat[3 * ec], nu = (T)A.mat[3 * ec + 1];
        rho = (T)A.mat[3 * ec + 2];
        mu = E / T(2.0) / (T(1.0) + nu);
        lambda = E * nu / (T(1.0) + nu) / (T(1.0) - T(2.0) * nu);
        const T Vp = sqrt((lambda + T(2.0) * mu) / rho);
        pm = (T)par[0]; L = (T)par[1];
        const T R = (T)par[2];
        const T lr = log(T(1.0) / R);
        a0 = (pm + T(1.0)) * (L / T(10.0)) / T(2.0) / L * lr;
        b0 = (pm + T(1.0)) * Vp / T(2.0) / L * lr;
        t = (T)((ND == 2 && A.thick) ? A.thick[ec] : 1.0);
#pragma unroll
        for (int i = 0; i < NEN * ND; ++i) X[i] = (T)(Xd[i] - Xd[i % ND]);
#pragma unroll
        for (int i = 0; i < ND; ++i) { xoff[i] = (T)(Xd[i] - par[3 + i]); nrm[i] = (T)par[3 + ND + i]; }
    }
    const T g = (T)0.577350269189626;       // GaussQuadrature.cpp:303-316
    // this lane's node dofs
    const double* u0 = nullptr;
    for (int k = 0; k < 4; ++k)
        if (A.coef_f[k] != 0.0f && !(ND == 2 && k == 3)) { u0 = A.u[k]; break; }
    T uq[NN];
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
        for (int i = 0; i < NN; ++i) uq[i] = u0 ? A.u_f[A.edof[(size_t)ec * NC + q * NN + i]] : 0.0f;
    } else {
#pragma unroll
        for (int i = 0; i < NN; ++i)
            uq[i] = u0 ? (T)(A.edof ? u0[A.edof[(size_t)ec * NC + q * NN + i]] : u0[(size_t)ec * NC + q * NN + i]) : T(0.0);
    }
    // Gauss point q
    const T xi[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, (q & 4) ? g : -g};
    T N[NEN], dN[NEN][3];
    if (ND == 2) {
        const T sr[4] = {-1, 1, 1, -1}, ss[4] = {-1, -1, 1, 1};
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            N[a] = T(0.25) * (T(1.0) + sr[a] * xi[0]) * (T(1.0) + ss[a] * xi[1]);
            dN[a][0] = T(0.25) * sr[a] * (T(1.0) + ss[a] * xi[1]);
            dN[a][1] = T(0.25) * ss[a] * (T(1.0) + sr[a] * xi[0]);
            dN[a][2] = T(0.0);
        }
    } else {
        const T sr[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, ss[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
        const T st[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
            const T fr = T(1.0) + sr[a] * xi[0], fs = T(1.0) + ss[a] * xi[1], ft = T(1.0) + st[a] * xi[2];
            N[a] = T(0.125) * fr * fs * ft;
            dN[a][0] = T(0.125) * sr[a] * fs * ft;
            dN[a][1] = T(0.125) * ss[a] * fr * ft;
            dN[a][2] = T(0.125) * st[a] * fr * fs;
        }
    }
    T J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, xg[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            xg[i] += N[a] * X[a * ND + i];
#pragma unroll
            for (int j = 0; j < ND; ++j) J[i][j] += dN[a][i] * X[a * ND + j];
        }
    T det, Ji[3][3];
    if (ND == 2) {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
        Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
    } else {
        const T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        Ji[0][0] = c00 / det;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        Ji[1][0] = c01 / det;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        Ji[2][0] = c02 / det;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    }
    T dx[NEN][3];
#pragma unroll
    for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T v = T(0.0);
            if (j < ND)
#pragma unroll
                for (int i = 0; i < ND; ++i) v += Ji[j][i] * dN[a][i];
            dx[a][j] = v;
        }
    const T f = ND == 2 ? t * fabs(det) : fabs(det);
    T as[3] = {1, 1, 1}, bs[3] = {0, 0, 0};
#pragma unroll
    for (int i = 0; i < ND; ++i) {
        const T r = pow((xoff[i] + xg[i]) * nrm[i] / L, pm);
        as[i] = T(1.0) + a0 * r;
        bs[i] = b0 * r;
    }
    // coefficient-weighted stretching combination of the active matrices
    T s = 0, qx = 0, qy = 0, qz = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        T ck;
        if constexpr (std::is_same<T, float>::value) ck = A.coef_f[k];
        else ck = A.coef[k];
        if (ck == T(0.0) || (ND == 2 && k == 3)) continue;
        T sk, xk, yk, zk = 0;
        if (ND == 2) {
            if (k == 0) { sk = as[0] * as[1]; xk = 0; yk = 0; }
            else if (k == 1) { sk = as[0] * bs[1] + as[1] * bs[0]; xk = as[1]; yk = as[0]; }
            else { sk = bs[0] * bs[1]; xk = bs[1]; yk = bs[0]; }
        } else {
            if (k == 0) { sk = as[0] * as[1] * as[2]; xk = yk = zk = 0; }
            else if (k == 1) {
                sk = as[0] * as[1] * bs[2] + as[0] * bs[1] * as[2] + bs[0] * as[1] * as[2];
                xk = as[1] * as[2]; yk = as[0] * as[2]; zk = as[0] * as[1];
            } else if (k == 2) {
                sk = as[0] * bs[1] * bs[2] + bs[0] * bs[1] * as[2] + bs[0] * as[1] * bs[2];
                xk = as[1] * bs[2] + as[2] * bs[1]; yk = as[0] * bs[2] + as[2] * bs[0]; zk = as[0] * bs[1] + as[1] * bs[0];
            } else {
                sk = bs[0] * bs[1] * bs[2];
                xk = bs[1] * bs[2]; yk = bs[0] * bs[2]; zk = bs[0] * bs[1];
            }
        }
        s += ck * sk; qx += ck * xk; qy += ck * yk; qz += ck * zk;
    }
    // interpolated displacement, stress and displacement gradient at this point
    T U[3] = {0, 0, 0}, S[NS], Gd[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int i = 0; i < NS; ++i) S[i] = T(0.0);
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const T ua = __shfl_sync(0xffffffffu, uq[d], base + a);
            U[d] += N[a] * ua;
#pragma unroll
            for (int j = 0; j < ND; ++j) Gd[d][j] += ua * dx[a][j];
        }
#pragma unroll
        for (int i = 0; i < NS; ++i) S[i] += N[a] * __shfl_sync(0xffffffffu, uq[ND + i], base + a);
    }
    T y[NC];
#pragma unroll
    for (int j = 0; j < NEN; ++j) {
        const T Nj = N[j];
        T* yj = y + j * NN;
        if (ND == 2) {
            const T k2 = s * (lambda + T(2.0) * mu) / T(4.0) / mu / (lambda + mu);
            const T l2 = s * lambda / T(4.0) / mu / (lambda + mu);
            yj[0] = f * (rho * s * Nj * U[0] + qx * dx[j][0] * S[0] + qy * dx[j][1] * S[2]);
            yj[1] = f * (rho * s * Nj * U[1] + qy * dx[j][1] * S[1] + qx * dx[j][0] * S[2]);
            yj[2] = f * Nj * (-k2 * S[0] + l2 * S[1] + qx * Gd[0][0]);
            yj[3] = f * Nj * (-k2 * S[1] + l2 * S[0] + qy * Gd[1][1]);
            yj[4] = f * Nj * (-s / mu * S[2] + qy * Gd[0][1] + qx * Gd[1][0]);
        } else {
            const T kap = s * (lambda + mu) / mu / (T(3.0) * lambda + T(2.0) * mu);
            const T lam = s * lambda / T(2.0) / mu / (T(3.0) * lambda + T(2.0) * mu);
            const T dxj = dx[j][0], dyj = dx[j][1], dzj = dx[j][2];
            yj[0] = f * (rho * s * Nj * U[0] + qx * dxj * S[0] + qy * dyj * S[3] + qz * dzj * S[5]);
            yj[1] = f * (rho * s * Nj * U[1] + qy * dyj * S[1] + qx * dxj * S[3] + qz * dzj * S[4]);
            yj[2] = f * (rho * s * Nj * U[2] + qz * dzj * S[2] + qx * dxj * S[5] + qy * dyj * S[4]);
            yj[3] = f * Nj * (-kap * S[0] + lam * (S[1] + S[2]) + qx * Gd[0][0]);
            yj[4] = f * Nj * (-kap * S[1] + lam * (S[0] + S[2]) + qy * Gd[1][1]);
            yj[5] = f * Nj * (-kap * S[2] + lam * (S[0] + S[1]) + qz * Gd[2][2]);
            yj[6] = f * Nj * (-s / mu * S[3] + qy * Gd[0][1] + qx * Gd[1][0]);
            yj[7] = f * Nj * (-s / mu * S[4] + qz * Gd[1][2] + qy * Gd[2][1]);
            yj[8] = f * Nj * (-s / mu * S[5] + qz * Gd[0][2] + qx * Gd[2][0]);
        }
    }
#pragma unroll
    for (int off = 1; off < NEN; off <<= 1)
#pragma unroll
        for (int j = 0; j < NC; ++j) y[j] += __shfl_xor_sync(0xffffffffu, y[j], off);
    if (!valid) return;
    if constexpr (std::is_same<T, float>::value) {
        float* outf = A.y_f + (size_t)ec * NC + q * NN;
#pragma unroll
        for (int i = 0; i < NN; ++i) {
            T mine = 0;
#pragma unroll
            for (int a = 0; a < NEN; ++a)
                if (a == q) mine = y[a * NN + i];
            outf[i] = mine;
        }
        return;
    }
    double* out = A.y + (size_t)ec * NC + q * NN;
#pragma unroll
    for (int i = 0; i < NN; ++i) {
        T mine = 0;
#pragma unroll
        for (int a = 0; a < NEN; ++a)
            if (a == q) mine = y[a * NN + i];
        double v = (double)mine;
        if (A.ftol >= 0.0 && !(fabs(v) > A.ftol)) v = 0.0;
        v *= A.yscale;
        out[i] = A.accumulate ? out[i] + v : v;
    }
}

void pml_tab_fill(int nd, int nelem, const double* X, const double* mat, const double* thick, const double* par,
                  std::vector<float>& tab) {
    const int nen = nd == 2 ? 4 : 8, npar = 3 + 2 * nd, st = pml_tab_stride(nd);
    tab.assign((size_t)nelem * st, 0.0f);
    for (int e = 0; e < nelem; ++e) {
        float* t = &tab[(size_t)e * st];
        const double* x = X + (size_t)e * nen * nd;
        const double* p = par + (size_t)e * npar;
        for (int i = 0; i < nen * nd; ++i) t[i] = (float)(x[i] - x[i % nd]);
        for (int i = 0; i < nd; ++i) { t[nen * nd + i] = (float)(x[i] - p[3 + i]); t[nen * nd + nd + i] = (float)p[3 + nd + i]; }
        const double E = mat[3 * e], nu = mat[3 * e + 1], rho = mat[3 * e + 2];
        const double mu = E / 2.0 / (1 + nu), lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
        const double Vp = std::sqrt((lambda + 2.0 * mu) / rho);
        const double m = p[0], L = p[1], R = p[2];
        float* c = t + nen * nd + 2 * nd;
        c[0] = (float)mu; c[1] = (float)lambda; c[2] = (float)rho;
        c[3] = (float)((m + 1.0) * (L / 10.0) / 2.0 / L * std::log(1.0 / R));
        c[4] = (float)((m + 1.0) * Vp / 2.0 / L * std::log(1.0 / R));
        c[5] = (float)m; c[6] = (float)L; c[7] = (float)((nd == 2 && thick) ? thick[e] : 1.0);
    }
}

int pml_action_launch(int ndim, const PmlArgs& A, cudaStream_t st) {
    if (A.nelem <= 0) return SVL_OK;
    const int tb = 128, gb = (A.nelem + tb - 1) / tb;
    // one input vector for every active matrix (an operator application):
    // the Gauss-point-parallel form
    bool one = true;
    const double* u0 = nullptr;
    for (int k = 0; k < 4; ++k) {
        if (A.coef[k] == 0.0 || (ndim == 2 && k == 3)) continue;
        if (!u0) u0 = A.u[k];
        else if (A.u[k] != u0) one = false;
    }
    if (one && A.edof && (!A.single || (A.tab && A.u_f && A.y_f))) {
        const int nen = ndim == 2 ? 4 : 8;
        const int gg = (int)(((int64_t)A.nelem * nen + tb - 1) / tb);
        PmlArgs B = A;
        for (int k = 0; k < 4; ++k) B.coef_f[k] = (float)A.coef[k];
        if (A.single) {
            if (ndim == 2) k_pml_action_gp<2, float><<<gg, tb, 0, st>>>(B);
            else k_pml_action_gp<3, float><<<gg, tb, 0, st>>>(B);
        } else {
            if (ndim == 2) k_pml_action_gp<2, double><<<gg, tb, 0, st>>>(B);
            else k_pml_action_gp<3, double><<<gg, tb, 0, st>>>(B);
        }
        PML_TRY(cudaGetLastError());
        return SVL_OK;
    }
    if (A.single) {
        if (ndim == 2) k_pml_action<2, float><<<gb, tb, 0, st>>>(A);
        else k_pml_action<3, float><<<gb, tb, 0, st>>>(A);
    } else {
        if (ndim == 2) k_pml_action<2, double><<<gb, tb, 0, st>>>(A);
        else k_pml_action<3, double><<<gb, tb, 0, st>>>(A);
    }
    PML_TRY(cudaGetLastError());
    return SVL_OK;
}

}  // namespace svl

extern "C" int svl_pml_element_action(int32_t ndim, int32_t nelem, const double* X, const double* mat,
                                      const double* thick, const double* par, const double* coef,
                                      const double* u, double* y) {
    if ((ndim != 2 && ndim != 3) || nelem < 0 || !X || !mat || !par || !coef || !u || !y) {
        set_error("bad argument to svl_pml_element_action");
        return SVL_ERR_INVALID;
    }
    if (nelem == 0) return SVL_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error("no CUDA device available"); return SVL_ERR_NODEVICE; }
    const int nen = ndim == 2 ? 4 : 8, nn = ndim == 2 ? 5 : 9, nc = nen * nn, npar = 3 + 2 * ndim;
    const size_t E = (size_t)nelem;
    cudaStream_t st = nullptr;
    PML_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    std::vector<void*> bufs;
    int rc = SVL_OK;
    auto dev = [&](const double* h, size_t n) -> double* {
        void* p = nullptr;
        if (rc || cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) { rc = rc ? rc : SVL_ERR_NOMEM; return nullptr; }
        bufs.push_back(p);
        if (h && cudaMemcpyAsync(p, h, n * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess) rc = SVL_ERR_CUDA;
        return (double*)p;
    };
    PmlArgs A{};
    A.nelem = nelem;
    A.ftol = -1.0; A.yscale = 1.0; A.accumulate = 0; A.edof = nullptr;
    A.X = dev(X, E * nen * ndim);
    A.mat = dev(mat, E * 3);
    A.thick = thick ? dev(thick, E) : nullptr;
    A.par = dev(par, E * npar);
    for (int i = 0; i < 4; ++i) {
        A.coef[i] = coef[i];
        A.u[i] = coef[i] != 0.0 ? dev(u + (size_t)i * E * nc, E * nc) : nullptr;
    }
    A.y = dev(nullptr, E * nc);
    if (!rc) rc = pml_action_launch(ndim, A, st);
    if (!rc && cudaMemcpyAsync(y, A.y, E * nc * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = SVL_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = SVL_ERR_CUDA;
    for (void* p : bufs) cudaFree(p);
    cudaStreamDestroy(st);
    if (rc == SVL_ERR_NOMEM) set_error("device allocation failed in svl_pml_element_action");
    else if (rc) set_error("CUDA error in svl_pml_element_action");
    return rc;
}
