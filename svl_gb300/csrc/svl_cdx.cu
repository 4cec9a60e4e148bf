// Mixed-precision batched central difference on uniform lin3DHexa8 grids.
//
// One fused kernel per step (k_cdx_step).  Each CTA owns a TX x TY x TZ block
// of nodes of one instance and
//   1. stages the (TX+2) x (TY+2) x (TZ+2) halo of FP64 displacements and the
//      lambda/mu of the (TX+1)(TY+1)(TZ+1) elements touching its nodes in
//      shared memory;
//   2. computes those elements' internal forces as a tcgen05 GEMM, 128
//      elements per MMA tile:  D[128 x 48] = U_e[128 x 24] . [K_lambda; K_mu]^T,
//      with TF32 hi/lo operands (hi.hi + hi.lo + lo.hi, FP32 accumulation in
//      TMEM), then F_e = lambda_e D[:, 0:24] + mu_e D[:, 24:48];
//   3. gathers the eight element contributions of every owned node in the
//      reference's element-tag order (no atomics) and updates
//      u_{n+1} = 2 u_n - u_{n-1} + (dt^2/m)(f_ext - f_int) in FP64
//      (CentralDifference.cpp:138-148 with the diagonal solve, for lumped
//      mass without damping).
// Element-local dof order and node order follow lin3DHexa8.cpp:756-853.
// A small k_cdx_loads kernel adds (dt^2/m) f_ext for the loaded dofs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "svl_internal.hpp"

using namespace svl;

namespace {

#define CUDA_TRY(x)                                                                  \
    do {                                                                             \
        cudaError_t err_ = (x);                                                      \
        if (err_ != cudaSuccess) {                                                   \
            set_error("%s failed: %s (%s:%d)", #x, cudaGetErrorString(err_), __FILE__, __LINE__); \
            return SVL_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)
#define TRY(x) do { int st_ = (x); if (st_ != SVL_OK) return st_; } while (0)

// Node tile owned by one CTA and derived sizes.
constexpr int TX = 8, TY = 8, TZ = 4;
constexpr int HX = TX + 2, HY = TY + 2, HZ = TZ + 2;          // halo nodes
constexpr int EX = TX + 1, EY = TY + 1, EZ = TZ + 1;          // elements touching the tile
constexpr int NEL = EX * EY * EZ;                             // 405
constexpr int NMT = (NEL + 127) / 128;                        // MMA tiles of 128 elements
constexpr int NTHREADS = 256;
constexpr int FSTRIDE = 25;                                   // padded row of element forces

// Canonical no-swizzle K-major operand layout: 8-row x 16-byte core matrices;
// element (r, k) at (r/8)*SBO + (k/4)*LBO + (r%8)*16 + (k%4)*4 bytes.
constexpr int KDIM = 24;                                      // element dofs
constexpr int LBO = 128;                                      // next core matrix along K
constexpr int SBO = (KDIM / 4) * 128;                         // next 8 rows: 768 B
constexpr int A_BYTES = (128 / 8) * SBO;                      // 12288 B per operand
constexpr int B_BYTES = (48 / 8) * SBO;                       // 4608 B per operand

// Shared memory carve-up (bytes, 1024-aligned operands first).
constexpr int OFF_AHI = 0;
constexpr int OFF_ALO = OFF_AHI + A_BYTES;
constexpr int OFF_BHI = OFF_ALO + A_BYTES;
constexpr int OFF_BLO = OFF_BHI + 5120;                        // B_BYTES rounded to 1 KB
constexpr int OFF_U = OFF_BLO + 5120;
constexpr int OFF_LAM = OFF_U + HX * HY * HZ * 3 * 8;
constexpr int OFF_MU = OFF_LAM + NEL * 4;
constexpr int OFF_F = OFF_MU + NEL * 4;
constexpr int align_up(int x, int a) { return (x + a - 1) / a * a; }
constexpr int OFF_BAR = align_up(OFF_F + NEL * FSTRIDE * 4, 16);   // mbarrier: 8-byte aligned
constexpr int OFF_TMEM = OFF_BAR + 16;
constexpr int SMEM_BYTES = OFF_TMEM + 16;
static_assert(OFF_BAR % 8 == 0 && OFF_TMEM % 4 == 0, "barrier / TMEM slot alignment");
static_assert(OFF_AHI % 1024 == 0 && OFF_ALO % 1024 == 0 && OFF_BHI % 1024 == 0 && OFF_BLO % 1024 == 0,
              "MMA operands start on 1 KB boundaries");
static_assert(OFF_U % 8 == 0 && OFF_LAM % 4 == 0 && OFF_MU % 4 == 0 && OFF_F % 4 == 0, "staging alignment");

constexpr uint32_t TMEM_COLS = 64;
constexpr long kWaitLimit = 2000000;    // bounded mbarrier wait (well under a second)

// Instruction descriptor for tcgen05.mma.kind::tf32: D = F32 (bits 4-5),
// A = B = TF32 (bits 7-9, 10-12), both K-major, N >> 3 (bits 17-22),
// M >> 4 (bits 24-28).
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((48u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (no swizzle, version 1).
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(LBO >> 4) << 16) |
           ((uint64_t)(SBO >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ float to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (long it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct CdxView {
    int nx, ny, nz, ninst;
    long long nn, ne;                // nodes / elements per instance
    const double* __restrict__ ucur; // [inst][node][3]
    double* uprev;                   // read u_{n-1}, write u_{n+1} (same node, same thread)
    const float* __restrict__ lam;   // [inst][element]
    const float* __restrict__ mu;
    const float* __restrict__ cdof;  // [inst][node][3]  dt^2/m, 0 on restrained dofs
    const float* __restrict__ bop;   // [2][B_BYTES/4] hi, lo operand images
    int* step;
    int* status;
};

__global__ void __launch_bounds__(NTHREADS, 2) k_cdx_step(CdxView v) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int ntz = (v.nz + 1 + TZ - 1) / TZ;
    const int inst = blockIdx.z / ntz;
    const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = (blockIdx.z % ntz) * TZ;
    const int nxn = v.nx + 1, nyn = v.ny + 1, nzn = v.nz + 1;
    if (tid == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) v.step[0] += 1;

    double* sU = reinterpret_cast<double*>(smem + OFF_U);
    float* sLam = reinterpret_cast<float*>(smem + OFF_LAM);
    float* sMu = reinterpret_cast<float*>(smem + OFF_MU);
    float* sF = reinterpret_cast<float*>(smem + OFF_F);
    float* sAhi = reinterpret_cast<float*>(smem + OFF_AHI);
    float* sAlo = reinterpret_cast<float*>(smem + OFF_ALO);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + OFF_TMEM);

    // -- TMEM allocation (warp 0) and the MMA barrier ------------------------
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(tmem_slot)), "r"(TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(bar)) : "memory");
    }

    // -- stage B operands, displacement halo and lambda/mu ------------------
    {
        const float4* src = reinterpret_cast<const float4*>(v.bop);
        float4* dhi = reinterpret_cast<float4*>(smem + OFF_BHI);
        float4* dlo = reinterpret_cast<float4*>(smem + OFF_BLO);
        for (int i = tid; i < B_BYTES / 16; i += NTHREADS) {
            dhi[i] = src[i];
            dlo[i] = src[B_BYTES / 16 + i];
        }
    }
    const double* ug = v.ucur + (size_t)inst * v.nn * 3;
    for (int i = tid; i < HX * HY * HZ * 3; i += NTHREADS) {
        const int c = i % 3, hn = i / 3;
        const int hx = hn % HX, hy = (hn / HX) % HY, hz = hn / (HX * HY);
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy, gz = z0 - 1 + hz;
        double val = 0.0;
        if (gx >= 0 && gx < nxn && gy >= 0 && gy < nyn && gz >= 0 && gz < nzn)
            val = ug[(((size_t)gz * nyn + gy) * nxn + gx) * 3 + c];
        sU[i] = val;
    }
    for (int le = tid; le < NEL; le += NTHREADS) {
        const int lx = le % EX, ly = (le / EX) % EY, lz = le / (EX * EY);
        const int ex = x0 - 1 + lx, ey = y0 - 1 + ly, ez = z0 - 1 + lz;
        float l = 0.f, m = 0.f;
        if (ex >= 0 && ex < v.nx && ey >= 0 && ey < v.ny && ez >= 0 && ez < v.nz) {
            const size_t g = (size_t)inst * v.ne + ((size_t)ez * v.ny + ey) * v.nx + ex;
            l = v.lam[g];
            m = v.mu[g];
        }
        sLam[le] = l;
        sMu[le] = m;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t bar_a = smem_u32(bar);
    bool ok = true;

    // -- element forces, one 128-element MMA tile at a time ----------------
    for (int t = 0; t < NMT; ++t) {
        {   // build A rows: thread pair per element, 4 nodes (12 dofs) each
            const int m = tid >> 1, half = tid & 1;
            const int le = t * 128 + m;
            float hi[12], lo[12];
            if (le < NEL) {
                const int lx = le % EX, ly = (le / EX) % EY, lz = le / (EX * EY);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int a = half * 4 + q;
                    // lin3DHexa8 node offsets: n1..n8
                    const int dx = (a == 1 || a == 2 || a == 5 || a == 6) ? 1 : 0;
                    const int dy = (a == 2 || a == 3 || a == 6 || a == 7) ? 1 : 0;
                    const int dz = (a >= 4) ? 1 : 0;
                    const int hn = ((lz + dz) * HY + (ly + dy)) * HX + (lx + dx);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const double u = sU[hn * 3 + c];
                        const float h = to_tf32(__double2float_rn(u));
                        hi[q * 3 + c] = h;
                        lo[q * 3 + c] = to_tf32(__double2float_rn(u - (double)h));
                    }
                }
            } else {
#pragma unroll
                for (int i = 0; i < 12; ++i) { hi[i] = 0.f; lo[i] = 0.f; }
            }
#pragma unroll
            for (int i = 0; i < 12; ++i) {
                const int k = half * 12 + i;
                const int off = (m >> 3) * (SBO / 4) + (k >> 2) * (LBO / 4) + (m & 7) * 4 + (k & 3);
                sAhi[off] = hi[i];
                sAlo[off] = lo[i];
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a_hi = smem_u32(smem + OFF_AHI), a_lo = smem_u32(smem + OFF_ALO);
            const uint32_t b_hi = smem_u32(smem + OFF_BHI), b_lo = smem_u32(smem + OFF_BLO);
            uint32_t acc = 0;
#pragma unroll
            for (int ks = 0; ks < KDIM / 8; ++ks) {           // three K=8 steps (2 core matrices each)
                const uint32_t koff = ks * 2 * LBO;
                mma_tf32(tmem, make_desc(a_hi + koff), make_desc(b_hi + koff), acc); acc = 1;
                mma_tf32(tmem, make_desc(a_hi + koff), make_desc(b_lo + koff), 1);
                mma_tf32(tmem, make_desc(a_lo + koff), make_desc(b_hi + koff), 1);
            }
            mma_commit(bar_a);
        }
        __syncwarp();
        ok = mbar_wait(bar_a, (uint32_t)(t & 1));
        ok = __syncthreads_and(ok) != 0;          // keep the .sync.aligned loads warp-uniform
        if (!ok && tid == 0) atomicOr(v.status, 1);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (warp < 4 && ok) {
            float d[48];
            const uint32_t row = tmem + ((uint32_t)(warp * 32) << 16);
            tmem_ld16(row + 0, d);
            tmem_ld16(row + 16, d + 16);
            tmem_ld16(row + 32, d + 32);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int le = t * 128 + warp * 32 + lane;
            if (le < NEL) {
                const float l = sLam[le], m = sMu[le];
#pragma unroll
                for (int j = 0; j < 24; ++j) sF[le * FSTRIDE + j] = l * d[j] + m * d[24 + j];
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (!ok) break;
    }

    // -- ordered gather and FP64 update of the owned nodes ------------------
    if (ok) {
        const int ox = tid % TX, oy = (tid / TX) % TY, oz = tid / (TX * TY);   // 256 = TX*TY*TZ
        const int gx = x0 + ox, gy = y0 + oy, gz = z0 + oz;
        if (gx < nxn && gy < nyn && gz < nzn) {
            // (element offset, local node) in ascending element-tag order
            const int sel[8][4] = {{0, 0, 0, 6}, {1, 0, 0, 7}, {0, 1, 0, 5}, {1, 1, 0, 4},
                                   {0, 0, 1, 2}, {1, 0, 1, 3}, {0, 1, 1, 1}, {1, 1, 1, 0}};
            float f[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                const int le = ((oz + sel[s][2]) * EY + (oy + sel[s][1])) * EX + (ox + sel[s][0]);
                const float* fe = sF + le * FSTRIDE + sel[s][3] * 3;
                f[0] += fe[0]; f[1] += fe[1]; f[2] += fe[2];
            }
            const size_t node = ((size_t)gz * nyn + gy) * nxn + gx;
            const size_t base = ((size_t)inst * v.nn + node) * 3;
            const int hn = ((oz + 1) * HY + (oy + 1)) * HX + (ox + 1);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double u = sU[hn * 3 + c];
                const double up = v.uprev[base + c];
                const double cc = (double)v.cdof[base + c];
                v.uprev[base + c] = (u + (u - up)) - cc * (double)f[c];
            }
        }
    }

    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// u_{n+1} += (dt^2/m) f_ext(k) on the loaded dofs (one thread per dof,
// entries of a dof summed in input order).
__global__ void k_cdx_loads(double* unext, const float* __restrict__ cdof, int nld, const long long* __restrict__ ld_dof,
                            const int* __restrict__ ld_ptr, const int* __restrict__ ld_ser, const double* __restrict__ ld_coef,
                            const int* __restrict__ s_ptr, const double* __restrict__ s_val, const int* step) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nld) return;
    const int k = step[0];
    double f = 0.0;
    for (int j = ld_ptr[i]; j < ld_ptr[i + 1]; ++j) {
        const int s = ld_ser[j];
        const int b = s_ptr[s], n = s_ptr[s + 1] - b;
        f += ld_coef[j] * ((k >= 0 && k < n) ? s_val[b + k] : 0.0);
    }
    const long long d = ld_dof[i];
    unext[d] += (double)cdof[d] * f;
}

// V and A of the last step from u_{n+1}, u_n, u_{n-1} (CentralDifference.cpp:141-144).
__global__ void k_cdx_va(const double* unext, const double* ucur, const double* uprev_copy, double* V, double* A,
                         long long n, double inv_2dt, double inv_dt2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double un = unext[i], u = ucur[i], up = uprev_copy[i];
    const double dU = un - u;
    V[i] = inv_2dt * (u + dU - up);
    A[i] = inv_dt2 * (dU - u + up);
}

float host_tf32(double x) {
    float f = (float)x;
    uint32_t b;
    std::memcpy(&b, &f, 4);
    if ((b & 0x7f800000u) != 0x7f800000u) b = (b + 0x1000u) & ~0x1FFFu;   // round to nearest, ties away
    float r;
    std::memcpy(&r, &b, 4);
    return r;
}

}  // namespace

struct svl_cdx {
    int nx = 0, ny = 0, nz = 0, ninst = 0;
    long long nn = 0, ne = 0, ntotal = 0;
    double dt = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    double* u[2] = {nullptr, nullptr};
    double* uprev_copy = nullptr;
    double* V = nullptr;
    double* A = nullptr;
    float *lam = nullptr, *mu = nullptr, *cdof = nullptr, *bop = nullptr;
    int *step = nullptr, *status = nullptr;
    long long* ld_dof = nullptr;
    int *ld_ptr = nullptr, *ld_ser = nullptr, *s_ptr = nullptr;
    double *ld_coef = nullptr, *s_val = nullptr;
    int nld = 0;
    int cur = 0;                     // index of u_n in u[]
    int64_t launches = 0, launches_last = 0;
    bool va_valid = false;

    template <typename T>
    int alloc(size_t n, T** out) {
        void* p = nullptr;
        const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        if (cudaMalloc(&p, bytes) != cudaSuccess) { set_error("cudaMalloc of %zu bytes failed", bytes); return SVL_ERR_NOMEM; }
        allocs.push_back(p);
        CUDA_TRY(cudaMemsetAsync(p, 0, bytes, stream));
        *out = static_cast<T*>(p);
        return SVL_OK;
    }
    template <typename T>
    int upload(const std::vector<T>& h, T** out) {
        TRY(alloc(h.size(), out));
        if (!h.empty()) CUDA_TRY(cudaMemcpyAsync(*out, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream));
        return SVL_OK;
    }
    ~svl_cdx() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }
};

static int cdx_check_instance(const svl_grid_spec* g, const HostModel& m, int inst) {
    const int nx = g->ne[0], ny = g->ne[1], nz = g->ne[2];
    const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    if (m.etype != SVL_ELEM_LIN3DHEXA8 || m.ndim != 3) { set_error("instance %d: the structured path needs lin3DHexa8", inst); return SVL_ERR_UNSUPPORTED; }
    if (m.nnode != nn || m.nelem != (long long)nx * ny * nz) { set_error("instance %d does not match the grid size", inst); return SVL_ERR_INVALID; }
    if (m.nconstraint) { set_error("instance %d: constraints are not supported on the structured path", inst); return SVL_ERR_UNSUPPORTED; }
    if (!m.lumped) { set_error("instance %d: the explicit path needs a lumped mass", inst); return SVL_ERR_UNSUPPORTED; }
    for (int k = 0; k < m.nmat; ++k)
        if (m.mtype[k] != SVL_MAT_ELASTIC3DLINEAR) { set_error("instance %d: only Elastic3DLinear on the structured path", inst); return SVL_ERR_UNSUPPORTED; }
    // node coordinates on the grid, PlainScheme total dofs 3n+c, generator connectivity
    for (long long n = 0; n < nn; ++n) {
        const int i = (int)(n % (nx + 1)), j = (int)((n / (nx + 1)) % (ny + 1)), k = (int)(n / ((long long)(nx + 1) * (ny + 1)));
        const double X[3] = {g->origin[0] + i * g->h[0], g->origin[1] + j * g->h[1], g->origin[2] + k * g->h[2]};
        for (int c = 0; c < 3; ++c) {
            if (std::fabs(m.X[n * 3 + c] - X[c]) > 1e-9 * (1.0 + std::fabs(X[c]))) { set_error("instance %d: node %lld is off the grid", inst, n); return SVL_ERR_INVALID; }
            if (m.tdof[n * 3 + c] != n * 3 + c) { set_error("instance %d: total dofs are not in PlainScheme grid order", inst); return SVL_ERR_INVALID; }
        }
    }
    const long long layer = (long long)(nx + 1) * (ny + 1);
    long long e = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i, ++e) {
                const long long n1 = layer * k + (long long)j * (nx + 1) + i;
                const long long want[8] = {n1, n1 + 1, n1 + 1 + (nx + 1), n1 + (nx + 1),
                                           n1 + layer, n1 + layer + 1, n1 + layer + 1 + (nx + 1), n1 + layer + (nx + 1)};
                for (int a = 0; a < 8; ++a)
                    if (m.conn[e * 8 + a] != want[a]) { set_error("instance %d: element %lld connectivity is not the grid's", inst, e); return SVL_ERR_INVALID; }
            }
    return SVL_OK;
}

extern "C" {

int svl_cdx_create(const svl_grid_spec* g, int32_t ninst, const svl_model_desc* models, const svl_load_desc* loads,
                   const svl_cd_opts* opts, svl_cdx** out) {
    if (!g || !models || !opts || !out || ninst <= 0) { set_error("NULL argument or ninst <= 0"); return SVL_ERR_INVALID; }
    *out = nullptr;
    if (g->ndim != 3) { set_error("the structured mixed path is 3D (lin3DHexa8)"); return SVL_ERR_UNSUPPORTED; }
    if (opts->precision != SVL_PREC_MIXED) { set_error("svl_cdx_create needs precision SVL_PREC_MIXED"); return SVL_ERR_UNSUPPORTED; }
    if (!(opts->dt > 0)) { set_error("dt must be positive"); return SVL_ERR_INVALID; }
    if (g->ne[0] <= 0 || g->ne[1] <= 0 || g->ne[2] <= 0) { set_error("bad grid"); return SVL_ERR_INVALID; }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error("no CUDA device available"); return SVL_ERR_NODEVICE; }
    svl_cdx* h = new svl_cdx();
    auto fail = [&](int st) { delete h; return st; };
    h->nx = g->ne[0]; h->ny = g->ne[1]; h->nz = g->ne[2]; h->ninst = ninst;
    h->nn = (long long)(h->nx + 1) * (h->ny + 1) * (h->nz + 1);
    h->ne = (long long)h->nx * h->ny * h->nz;
    h->ntotal = h->nn * 3;
    h->dt = opts->dt;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) { set_error("cudaStreamCreate failed"); return fail(SVL_ERR_CUDA); }

    std::vector<float> lam((size_t)ninst * h->ne), mu((size_t)ninst * h->ne), cdof((size_t)ninst * h->ntotal);
    std::vector<double> Klam(24 * 24, 0.0), Kmu(24 * 24, 0.0);
    const double dt2 = opts->dt * opts->dt;
    std::vector<long long> fdof;
    std::vector<int> fser;
    std::vector<double> fcoef;
    std::vector<int> s_ptr(1, 0);
    std::vector<double> s_val;
    for (int b = 0; b < ninst; ++b) {
        HostModel m;
        if (!model_from_desc(&models[b], m)) return fail(SVL_ERR_INVALID);
        int st = cdx_check_instance(g, m, b);
        if (st) return fail(st);
        // every element must have the geometry of element 0 (uniform grid)
        if (b == 0) {
            for (int q = 0; q < 8; ++q) {
                double dNx[8][3], N[8];
                const double w = gp_factor(m, 0, gp_geometry(m, 0, q, dNx, N));
                double div[24], B[6][24];
                for (int i = 0; i < 24; ++i) { div[i] = 0; for (int s = 0; s < 6; ++s) B[s][i] = 0; }
                for (int a = 0; a < 8; ++a) {
                    const double bx = dNx[a][0], by = dNx[a][1], bz = dNx[a][2];
                    div[3 * a] = bx; div[3 * a + 1] = by; div[3 * a + 2] = bz;
                    B[0][3 * a] = bx; B[1][3 * a + 1] = by; B[2][3 * a + 2] = bz;
                    B[3][3 * a] = by; B[3][3 * a + 1] = bx;
                    B[4][3 * a + 1] = bz; B[4][3 * a + 2] = by;
                    B[5][3 * a] = bz; B[5][3 * a + 2] = bx;
                }
                // C = lambda m m^T + mu diag(2,2,2,1,1,1)
                static const double D[6] = {2, 2, 2, 1, 1, 1};
                for (int i = 0; i < 24; ++i)
                    for (int j = 0; j < 24; ++j) {
                        Klam[i * 24 + j] += w * div[i] * div[j];
                        double s = 0;
                        for (int r = 0; r < 6; ++r) s += B[r][i] * D[r] * B[r][j];
                        Kmu[i * 24 + j] += w * s;
                    }
            }
        }
        for (int e = 0; e < m.nelem; ++e) {
            if (e % 97 == 0 || e == m.nelem - 1) {     // spot-check the uniform geometry
                double d0[8][3], d1[8][3], N[8];
                for (int q = 0; q < 8; q += 7) {
                    const double w0 = gp_geometry(m, 0, q, d0, N), w1 = gp_geometry(m, e, q, d1, N);
                    if (std::fabs(w0 - w1) > 1e-12 * std::fabs(w0)) { set_error("instance %d: grid is not uniform", b); return fail(SVL_ERR_UNSUPPORTED); }
                }
            }
            const double* p = m.param(e);
            const double E = p[0], nu = p[1];
            lam[(size_t)b * h->ne + e] = (float)(E * nu / (1.0 - 2.0 * nu) / (1.0 + nu));
            mu[(size_t)b * h->ne + e] = (float)(E / (2.0 * (1.0 + nu)));
        }
        std::vector<double> M;
        lumped_mass_diag(m, opts->mtol, M);
        for (long long t = 0; t < h->ntotal; ++t) {
            const bool fixed = m.fdof[t] < 0;
            if (!fixed && !(M[t] > 0)) { set_error("instance %d: free dof %lld has no mass", b, t); return fail(SVL_ERR_INVALID); }
            cdof[(size_t)b * h->ntotal + t] = fixed ? 0.0f : (float)(dt2 / M[t]);
        }
        if (loads) {
            const svl_load_desc& L = loads[b];
            if (L.nsupport > 0) { set_error("instance %d: support motion is not supported on the structured path", b); return fail(SVL_ERR_UNSUPPORTED); }
            const int soff = (int)s_ptr.size() - 1;
            for (int s = 0; s < L.nseries; ++s) {
                const int n = L.series_ptr[s + 1] - L.series_ptr[s];
                if (n < 0) { set_error("bad series_ptr"); return fail(SVL_ERR_INVALID); }
                s_val.insert(s_val.end(), L.series_val + L.series_ptr[s], L.series_val + L.series_ptr[s + 1]);
                s_ptr.push_back((int)s_val.size());
            }
            for (int i = 0; i < L.nforce; ++i) {
                if (L.force_dof[i] < 0 || L.force_dof[i] >= h->ntotal || L.force_series[i] < 0 || L.force_series[i] >= L.nseries) {
                    set_error("instance %d: load entry %d out of range", b, i); return fail(SVL_ERR_INVALID);
                }
                fdof.push_back((long long)b * h->ntotal + L.force_dof[i]);
                fser.push_back(soff + L.force_series[i]);
                fcoef.push_back(L.force_coef[i]);
            }
        }
    }
    // B operand images: rows 0-23 K_lambda, 24-47 K_mu, canonical K-major layout
    std::vector<float> bop(2 * (B_BYTES / 4), 0.f);
    for (int n = 0; n < 48; ++n)
        for (int k = 0; k < 24; ++k) {
            const double val = n < 24 ? Klam[n * 24 + k] : Kmu[(n - 24) * 24 + k];
            const float hi = host_tf32(val);
            const float lo = host_tf32(val - (double)hi);
            const int off = (n >> 3) * (SBO / 4) + (k >> 2) * (LBO / 4) + (n & 7) * 4 + (k & 3);
            bop[off] = hi;
            bop[B_BYTES / 4 + off] = lo;
        }
    // loads grouped by dof, input order kept within a dof
    std::vector<int> order(fdof.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b2) { return fdof[a] < fdof[b2]; });
    std::vector<long long> ld_dof;
    std::vector<int> ld_ptr(1, 0), ld_ser;
    std::vector<double> ld_coef;
    for (size_t i = 0; i < order.size(); ++i) {
        const int j = order[i];
        if (ld_dof.empty() || ld_dof.back() != fdof[j]) { if (!ld_dof.empty()) ld_ptr.push_back((int)ld_ser.size()); ld_dof.push_back(fdof[j]); }
        ld_ser.push_back(fser[j]);
        ld_coef.push_back(fcoef[j]);
    }
    if (!ld_dof.empty()) ld_ptr.push_back((int)ld_ser.size());
    h->nld = (int)ld_dof.size();

    int st;
    const size_t nt = (size_t)ninst * h->ntotal;
    if ((st = h->alloc(nt, &h->u[0])) || (st = h->alloc(nt, &h->u[1])) || (st = h->alloc(nt, &h->uprev_copy)) ||
        (st = h->alloc(nt, &h->V)) || (st = h->alloc(nt, &h->A)) || (st = h->upload(lam, &h->lam)) ||
        (st = h->upload(mu, &h->mu)) || (st = h->upload(cdof, &h->cdof)) || (st = h->upload(bop, &h->bop)) ||
        (st = h->alloc(2, &h->step)) || (st = h->alloc(1, &h->status)) || (st = h->upload(ld_dof, &h->ld_dof)) ||
        (st = h->upload(ld_ptr, &h->ld_ptr)) || (st = h->upload(ld_ser, &h->ld_ser)) || (st = h->upload(ld_coef, &h->ld_coef)) ||
        (st = h->upload(s_ptr, &h->s_ptr)) || (st = h->upload(s_val, &h->s_val)))
        return fail(st);
    if (cudaFuncSetAttribute(k_cdx_step, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess) {
        set_error("cannot set %d bytes of dynamic shared memory", SMEM_BYTES); return fail(SVL_ERR_CUDA);
    }
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) { set_error("upload failed"); return fail(SVL_ERR_CUDA); }
    *out = h;
    return SVL_OK;
}

int svl_cdx_set_initial(svl_cdx* h, int32_t inst, const double* U0, const double* V0, const double* A0) {
    if (!h || inst < 0 || inst >= h->ninst) { set_error("bad handle or instance"); return SVL_ERR_INVALID; }
    const size_t n = (size_t)h->ntotal;
    std::vector<double> U(n, 0.0), Up(n);
    if (U0) std::memcpy(U.data(), U0, n * 8);
    for (size_t i = 0; i < n; ++i) {
        const double v = V0 ? V0[i] : 0.0, a = A0 ? A0[i] : 0.0;
        Up[i] = U[i] - h->dt * v + h->dt * h->dt / 2.0 * a;
    }
    CUDA_TRY(cudaMemcpyAsync(h->u[h->cur] + inst * n, U.data(), n * 8, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->u[1 - h->cur] + inst * n, Up.data(), n * 8, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->va_valid = false;
    return SVL_OK;
}

static int cdx_step(svl_cdx* h, bool want_va) {
    CdxView v;
    v.nx = h->nx; v.ny = h->ny; v.nz = h->nz; v.ninst = h->ninst;
    v.nn = h->nn; v.ne = h->ne;
    v.ucur = h->u[h->cur];
    v.uprev = h->u[1 - h->cur];
    v.lam = h->lam; v.mu = h->mu; v.cdof = h->cdof; v.bop = h->bop;
    v.step = h->step; v.status = h->status;
    const size_t nt = (size_t)h->ninst * h->ntotal;
    if (want_va) CUDA_TRY(cudaMemcpyAsync(h->uprev_copy, v.uprev, nt * 8, cudaMemcpyDeviceToDevice, h->stream));
    const dim3 grid((h->nx + 1 + TX - 1) / TX, (h->ny + 1 + TY - 1) / TY, ((h->nz + 1 + TZ - 1) / TZ) * h->ninst);
    k_cdx_step<<<grid, NTHREADS, SMEM_BYTES, h->stream>>>(v);
    ++h->launches;
    if (h->nld > 0) {
        k_cdx_loads<<<(h->nld + 127) / 128, 128, 0, h->stream>>>(v.uprev, h->cdof, h->nld, h->ld_dof, h->ld_ptr, h->ld_ser,
                                                               h->ld_coef, h->s_ptr, h->s_val, h->step);
        ++h->launches;
    }
    if (want_va) {
        k_cdx_va<<<(unsigned)((nt + 255) / 256), 256, 0, h->stream>>>(v.uprev, v.ucur, h->uprev_copy, h->V, h->A, (long long)nt,
                                                                   1.0 / 2.0 / h->dt, 1.0 / h->dt / h->dt);
        ++h->launches;
    }
    CUDA_TRY(cudaGetLastError());
    h->cur = 1 - h->cur;
    return SVL_OK;
}

int svl_cdx_run(svl_cdx* h, int32_t k_first, int32_t nsteps, double* U_hist) {
    if (!h || nsteps < 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    const int64_t l0 = h->launches;
    const int kstart = k_first - 1;
    CUDA_TRY(cudaMemcpyAsync(h->step, &kstart, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    const size_t nt = (size_t)h->ninst * h->ntotal;
    for (int s = 0; s < nsteps; ++s) {
        TRY(cdx_step(h, s == nsteps - 1));
        if (U_hist) CUDA_TRY(cudaMemcpyAsync(U_hist + (size_t)s * nt, h->u[h->cur], nt * 8, cudaMemcpyDeviceToHost, h->stream));
    }
    h->va_valid = nsteps > 0;
    h->launches_last = h->launches - l0;
    int status = 0;
    CUDA_TRY(cudaMemcpyAsync(&status, h->status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (status) { set_error("tensor-core step timed out waiting for an MMA (status %d)", status); return SVL_ERR_CUDA; }
    return SVL_OK;
}

int svl_cdx_run_timed(svl_cdx* h, int32_t k_first, int32_t nsteps, float* ms) {
    if (!h || !ms) { set_error("bad argument"); return SVL_ERR_INVALID; }
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    const int kstart = k_first - 1;
    CUDA_TRY(cudaMemcpyAsync(h->step, &kstart, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    const int64_t l0 = h->launches;
    CUDA_TRY(cudaEventRecord(a, h->stream));
    for (int s = 0; s < nsteps; ++s) TRY(cdx_step(h, false));
    CUDA_TRY(cudaEventRecord(b, h->stream));
    CUDA_TRY(cudaEventSynchronize(b));
    CUDA_TRY(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    h->launches_last = h->launches - l0;
    h->va_valid = false;
    int status = 0;
    CUDA_TRY(cudaMemcpy(&status, h->status, sizeof(int), cudaMemcpyDeviceToHost));
    if (status) { set_error("tensor-core step timed out waiting for an MMA (status %d)", status); return SVL_ERR_CUDA; }
    return SVL_OK;
}

int svl_cdx_get(svl_cdx* h, int32_t inst, int32_t which, double* out) {
    if (!h || !out || inst < 0 || inst >= h->ninst) { set_error("bad argument"); return SVL_ERR_INVALID; }
    const double* src = which == 0 ? h->u[h->cur] : which == 1 ? h->V : which == 2 ? h->A : nullptr;
    if (!src) { set_error("which must be 0, 1 or 2"); return SVL_ERR_INVALID; }
    if (which != 0 && !h->va_valid) { set_error("V/A are only available after svl_cdx_run"); return SVL_ERR_INVALID; }
    CUDA_TRY(cudaMemcpyAsync(out, src + (size_t)inst * h->ntotal, h->ntotal * 8, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SVL_OK;
}

int svl_cdx_launch_count(svl_cdx* h, int64_t* launches) {
    if (!h || !launches) { set_error("bad argument"); return SVL_ERR_INVALID; }
    *launches = h->launches_last;
    return SVL_OK;
}

void svl_cdx_destroy(svl_cdx* h) { delete h; }

}  // extern "C"
