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

template <int ND>
__global__ void __launch_bounds__(128) k_pml_action(PmlArgs A) {
    constexpr int NEN = ND == 2 ? 4 : 8, NN = ND == 2 ? 5 : 9, NC = NEN * NN, NS = ND == 2 ? 3 : 6;
    constexpr int NPAR = 3 + 2 * ND;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.nelem) return;
    const double* X = A.X + (size_t)e * NEN * ND;
    const double E = A.mat[3 * e], nu = A.mat[3 * e + 1], rho = A.mat[3 * e + 2];
    const double t = (ND == 2 && A.thick) ? A.thick[e] : 1.0;
    const double* par = A.par + (size_t)e * NPAR;
    const double mu = E / 2.0 / (1 + nu);
    const double lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
    const double Vp = sqrt((lambda + 2.0 * mu) / rho);
    const double pm = par[0], L = par[1], R = par[2];
    const double a0 = (pm + 1.0) * (L / 10.0) / 2.0 / L * log(1.0 / R);
    const double b0 = (pm + 1.0) * Vp / 2.0 / L * log(1.0 / R);
    const double g = 0.577350269189626;       // GaussQuadrature.cpp:303-316
    double y[NC];
#pragma unroll
    for (int i = 0; i < NC; ++i) y[i] = 0.0;
    // all active matrices on one input vector: a single weighted pass
    bool fused = true;
    {
        const double* u0 = nullptr;
        for (int k = 0; k < 4; ++k) {
            if (A.coef[k] == 0.0 || (ND == 2 && k == 3)) continue;
            if (!u0) u0 = A.u[k];
            else if (A.u[k] != u0) fused = false;
        }
    }
    for (int q = 0; q < NEN; ++q) {
        const double xi[3] = {(q & 1) ? g : -g, (q & 2) ? g : -g, (q & 4) ? g : -g};
        double N[NEN], dN[NEN][3];
        if (ND == 2) {
            const double sr[4] = {-1, 1, 1, -1}, ss[4] = {-1, -1, 1, 1};
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                N[a] = 0.25 * (1.0 + sr[a] * xi[0]) * (1.0 + ss[a] * xi[1]);
                dN[a][0] = 0.25 * sr[a] * (1.0 + ss[a] * xi[1]);
                dN[a][1] = 0.25 * ss[a] * (1.0 + sr[a] * xi[0]);
                dN[a][2] = 0.0;
            }
        } else {
            const double sr[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, ss[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
            const double st[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
                const double fr = 1.0 + sr[a] * xi[0], fs = 1.0 + ss[a] * xi[1], ft = 1.0 + st[a] * xi[2];
                N[a] = 0.125 * fr * fs * ft;
                dN[a][0] = 0.125 * sr[a] * fs * ft;
                dN[a][1] = 0.125 * ss[a] * fr * ft;
                dN[a][2] = 0.125 * st[a] * fr * fs;
            }
        }
        double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, xg[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int i = 0; i < ND; ++i) {
                xg[i] += N[a] * X[a * ND + i];
#pragma unroll
                for (int j = 0; j < ND; ++j) J[i][j] += dN[a][i] * X[a * ND + j];
            }
        double det, Ji[3][3];
        if (ND == 2) {
            det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
            Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
            Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
        } else {
            const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
            const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
            const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
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
        double dx[NEN][3];
#pragma unroll
        for (int a = 0; a < NEN; ++a)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                double v = 0.0;
                if (j < ND)
#pragma unroll
                    for (int i = 0; i < ND; ++i) v += Ji[j][i] * dN[a][i];
                dx[a][j] = v;
            }
        const double f = ND == 2 ? t * 1.0 * fabs(det) : 1.0 * fabs(det);
        double as[3] = {1, 1, 1}, bs[3] = {0, 0, 0};
#pragma unroll
        for (int i = 0; i < ND; ++i) {
            const double r = pow((xg[i] - par[3 + i]) * par[3 + ND + i] / L, pm);
            as[i] = 1.0 + a0 * r;
            bs[i] = b0 * r;
        }
        // stretching combinations of matrix mi (see the header)
        auto combo = [&](int mi, double& s, double& qx, double& qy, double& qz) {
            qz = 0.0;
            if (ND == 2) {
                if (mi == 0) { s = as[0] * as[1]; qx = 0; qy = 0; }
                else if (mi == 1) { s = as[0] * bs[1] + as[1] * bs[0]; qx = as[1]; qy = as[0]; }
                else { s = bs[0] * bs[1]; qx = bs[1]; qy = bs[0]; }
            } else {
                if (mi == 0) { s = as[0] * as[1] * as[2]; qx = qy = qz = 0.0; }
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
            double c, s, qx, qy, qz;
            const double* ubase;
            if (fused) {
                c = 1.0; s = qx = qy = qz = 0.0;
                ubase = nullptr;
                for (int k = 0; k < 4; ++k) {
                    if (A.coef[k] == 0.0 || (ND == 2 && k == 3)) continue;
                    double sk, xk, yk, zk;
                    combo(k, sk, xk, yk, zk);
                    s += A.coef[k] * sk; qx += A.coef[k] * xk; qy += A.coef[k] * yk; qz += A.coef[k] * zk;
                    ubase = A.u[k];
                }
                if (!ubase) continue;
            } else {
                c = A.coef[mi];
                if (c == 0.0 || (ND == 2 && mi == 3)) continue;
                combo(mi, s, qx, qy, qz);
                ubase = A.u[mi];
            }
            const double* u = ubase + (A.edof ? 0 : (size_t)e * NC);
            const int32_t* ed = A.edof ? A.edof + (size_t)e * NC : nullptr;
            // interpolated displacement, stress and displacement gradient
            double U[3] = {0, 0, 0}, S[NS], Gd[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
            for (int i = 0; i < NS; ++i) S[i] = 0.0;
#pragma unroll
            for (int a = 0; a < NEN; ++a) {
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const double ua = ed ? u[ed[a * NN + d]] : u[a * NN + d];
                    U[d] += N[a] * ua;
#pragma unroll
                    for (int j = 0; j < ND; ++j) Gd[d][j] += ua * dx[a][j];
                }
#pragma unroll
                for (int i = 0; i < NS; ++i) S[i] += N[a] * (ed ? u[ed[a * NN + ND + i]] : u[a * NN + ND + i]);
            }
            const double cf = c * f;
#pragma unroll
            for (int j = 0; j < NEN; ++j) {
                const double Nj = N[j];
                double* yj = y + j * NN;
                if (ND == 2) {
                    // dofs: ux uy s11 s22 s12
                    const double k2 = s * (lambda + 2.0 * mu) / 4.0 / mu / (lambda + mu);
                    const double l2 = s * lambda / 4.0 / mu / (lambda + mu);
                    yj[0] += cf * (rho * s * Nj * U[0] + qx * dx[j][0] * S[0] + qy * dx[j][1] * S[2]);
                    yj[1] += cf * (rho * s * Nj * U[1] + qy * dx[j][1] * S[1] + qx * dx[j][0] * S[2]);
                    yj[2] += cf * Nj * (-k2 * S[0] + l2 * S[1] + qx * Gd[0][0]);
                    yj[3] += cf * Nj * (-k2 * S[1] + l2 * S[0] + qy * Gd[1][1]);
                    yj[4] += cf * Nj * (-s / mu * S[2] + qy * Gd[0][1] + qx * Gd[1][0]);
                } else {
                    // dofs: ux uy uz s11 s22 s33 s12 s23 s13
                    const double kap = s * (lambda + mu) / mu / (3.0 * lambda + 2.0 * mu);
                    const double lam = s * lambda / 2.0 / mu / (3.0 * lambda + 2.0 * mu);
                    const double dxj = dx[j][0], dyj = dx[j][1], dzj = dx[j][2];
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
        double v = y[i];
        if (A.ftol >= 0.0 && !(fabs(v) > A.ftol)) v = 0.0;
        v *= A.yscale;
        out[i] = A.accumulate ? out[i] + v : v;
    }
}

int pml_action_launch(int ndim, const PmlArgs& A, cudaStream_t st) {
    if (A.nelem <= 0) return SVL_OK;
    const int tb = 128, gb = (A.nelem + tb - 1) / tb;
    if (ndim == 2) k_pml_action<2><<<gb, tb, 0, st>>>(A);
    else k_pml_action<3><<<gb, tb, 0, st>>>(A);
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
