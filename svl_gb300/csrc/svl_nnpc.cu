// Learned preconditioner kernels: 3x3x3 convolutions on the node lattice
// (forward, data gradient, weight gradient), loss, Adam, and the maps between
// free-dof vectors and lattice grids.  FP32 on the CUDA cores; every
// reduction runs in a fixed order, so training and inference are bitwise
// reproducible.  Interface and network in svl_nnpc.hpp.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "svl_internal.hpp"
#include "svl_nnpc.hpp"

namespace svl {

namespace {

#define NN_TRY(x)                                                                         \
    do {                                                                                  \
        cudaError_t err_ = (x);                                                           \
        if (err_ != cudaSuccess) {                                                        \
            set_error("%s failed: %s (%s:%d)", #x, cudaGetErrorString(err_), __FILE__, __LINE__); \
            return SVL_ERR_CUDA;                                                          \
        }                                                                                 \
    } while (0)

constexpr int kThreads = 256;
constexpr int kWgTile = 64;       // voxels per shared-memory tile of the weight gradient
constexpr int kWgChunk = 2048;    // voxels per block of the weight gradient
constexpr int kRedBlocks = 256;   // blocks of the loss reduction

struct Dims {
    int nx, ny, nz, V;
};

// out[co][v] = sum_{ci,t} W[co][ci][t] in[ci][v + s_t]   (s_t = tap offset, zero outside)
// optionally relu, optionally multiplied by (gate[co][v] > 0).
template <int CIN, int COUT, bool RELU>
__global__ void __launch_bounds__(kThreads) k_conv(const float* __restrict__ in, const float* __restrict__ W,
                                                   float* __restrict__ out, Dims d, const float* __restrict__ gate) {
    __shared__ float sw[COUT * CIN * kNnTaps];
    for (int i = threadIdx.x; i < COUT * CIN * kNnTaps; i += blockDim.x) sw[i] = W[i];
    __syncthreads();
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= d.V) return;
    const int x = v % d.nx, y = (v / d.nx) % d.ny, z = v / (d.nx * d.ny);
    const size_t V = (size_t)d.V;
    float acc[COUT];
#pragma unroll
    for (int co = 0; co < COUT; ++co) acc[co] = 0.f;
    for (int dz = -1; dz <= 1; ++dz) {
        if (z + dz < 0 || z + dz >= d.nz) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            if (y + dy < 0 || y + dy >= d.ny) continue;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                if (x + dx < 0 || x + dx >= d.nx) continue;
                const int t = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
                const size_t nb = (size_t)v + dx + (ptrdiff_t)dy * d.nx + (ptrdiff_t)dz * d.nx * d.ny;
#pragma unroll
                for (int ci = 0; ci < CIN; ++ci) {
                    const float a = __ldg(in + ci * V + nb);
#pragma unroll
                    for (int co = 0; co < COUT; ++co) acc[co] = fmaf(sw[(co * CIN + ci) * kNnTaps + t], a, acc[co]);
                }
            }
        }
    }
#pragma unroll
    for (int co = 0; co < COUT; ++co) {
        float r = RELU ? fmaxf(acc[co], 0.f) : acc[co];
        if (gate && !(gate[co * V + v] > 0.f)) r = 0.f;
        out[co * V + v] = r;
    }
}

// Wt[ci][co][26 - t] = W[co][ci][t]: the data gradient is a forward
// convolution of the output gradient with these weights.
__global__ void k_flip(const float* __restrict__ W, float* __restrict__ Wt, int cin, int cout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cin * cout * kNnTaps) return;
    const int t = i % kNnTaps, ci = (i / kNnTaps) % cin, co = i / (kNnTaps * cin);
    Wt[(ci * cout + co) * kNnTaps + (kNnTaps - 1 - t)] = W[i];
}

// partial[blk][t][co*CIN+ci] = sum over this block's voxels v of g[co][v] * a[ci][v + s_t]
template <int CIN, int COUT>
__global__ void __launch_bounds__(kThreads) k_wgrad(const float* __restrict__ g, const float* __restrict__ a,
                                                    float* __restrict__ partial, Dims d) {
    __shared__ float sg[COUT][kWgTile];
    __shared__ float sa[CIN][kWgTile];
    const int t = blockIdx.y;
    const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
    const int co = threadIdx.x / CIN, ci = threadIdx.x % CIN;
    const bool active = threadIdx.x < CIN * COUT;
    const size_t V = (size_t)d.V;
    const int v0 = blockIdx.x * kWgChunk, v1 = min(v0 + kWgChunk, d.V);
    float acc = 0.f;
    for (int base = v0; base < v1; base += kWgTile) {
        for (int i = threadIdx.x; i < (COUT + CIN) * kWgTile; i += blockDim.x) {
            const int c = i / kWgTile, j = i % kWgTile, v = base + j;
            float val = 0.f;
            if (v < v1) {
                if (c < COUT) {
                    val = g[c * V + v];
                } else {
                    const int x = v % d.nx, y = (v / d.nx) % d.ny, z = v / (d.nx * d.ny);
                    if (x + dx >= 0 && x + dx < d.nx && y + dy >= 0 && y + dy < d.ny && z + dz >= 0 && z + dz < d.nz)
                        val = a[(c - COUT) * V + v + dx + (ptrdiff_t)dy * d.nx + (ptrdiff_t)dz * d.nx * d.ny];
                }
            }
            if (c < COUT) sg[c][j] = val; else sa[c - COUT][j] = val;
        }
        __syncthreads();
        if (active) {
#pragma unroll 8
            for (int j = 0; j < kWgTile; ++j) acc = fmaf(sg[co][j], sa[ci][j], acc);
        }
        __syncthreads();
    }
    if (active) partial[((size_t)blockIdx.x * kNnTaps + t) * (CIN * COUT) + threadIdx.x] = acc;
}

// dW[(co*cin+ci)*27 + t] += sum over blocks (fixed order)
__global__ void k_wgrad_reduce(const float* __restrict__ partial, float* __restrict__ dW, int cin, int cout, int nblk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = cin * cout * kNnTaps;
    if (i >= n) return;
    const int t = i % kNnTaps, p = i / kNnTaps;     // p = co*cin + ci
    float s = 0.f;
    for (int b = 0; b < nblk; ++b) s += partial[((size_t)b * kNnTaps + t) * (cin * cout) + p];
    dW[i] += s;
}

// features [x ; rho * x] from a 3-channel grid
__global__ void k_feat_grid(const float* __restrict__ x, const float* __restrict__ rho, float* __restrict__ f, int n3) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n3) return;
    const float v = x[i];
    f[i] = v;
    f[n3 + i] = rho[i] * v;
}

// dst[c][k][j][i] = src[c][oz + k][oy + j][ox + i], c < 3: a window of a
// lattice grid (training on crops)
__global__ void k_crop(const float* __restrict__ src, float* __restrict__ dst, Dims full, Dims cr, int ox, int oy, int oz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * cr.V) return;
    const int c = i / cr.V, v = i % cr.V;
    const int x = v % cr.nx, y = (v / cr.nx) % cr.ny, z = v / (cr.nx * cr.ny);
    dst[i] = src[(size_t)c * full.V + ((size_t)(oz + z) * full.ny + (oy + y)) * full.nx + (ox + x)];
}

// loss mask of a window: the lattice mask, zero within `margin` voxels of a
// window face that lies inside the lattice (there the zero padding of the
// window differs from the lattice's neighbours; 4 = the network's reach)
__global__ void k_crop_mask(const float* __restrict__ mask, float* __restrict__ dst, Dims full, Dims cr, int ox, int oy,
                            int oz, int margin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * cr.V) return;
    const int c = i / cr.V, v = i % cr.V;
    const int x = v % cr.nx, y = (v / cr.nx) % cr.ny, z = v / (cr.nx * cr.ny);
    float m = mask[(size_t)c * full.V + ((size_t)(oz + z) * full.ny + (oy + y)) * full.nx + (ox + x)];
    if ((ox > 0 && x < margin) || (ox + cr.nx < full.nx && x >= cr.nx - margin) ||
        (oy > 0 && y < margin) || (oy + cr.ny < full.ny && y >= cr.ny - margin) ||
        (oz > 0 && z < margin) || (oz + cr.nz < full.nz && z >= cr.nz - margin))
        m = 0.f;
    dst[i] = m;
}

// features from a free-dof residual (grid pre-zeroed)
__global__ void k_feat_free(const double* __restrict__ r, const double* __restrict__ sdinv,
                            const float* __restrict__ rho_grid, const int32_t* __restrict__ gmap, float* __restrict__ f,
                            int nf, int n3) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const int g = gmap[i];
    const float v = (float)(r[i] * sdinv[i]);
    f[g] = v;
    f[n3 + g] = rho_grid[g] * v;
}

// z_f = D^-1/2 (r_hat_f + y[gmap f])
__global__ void k_out_free(const float* __restrict__ y, const double* __restrict__ r, const double* __restrict__ sdinv,
                           const int32_t* __restrict__ gmap, double* __restrict__ z, int nf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const double s = sdinv[i];
    z[i] = s * (r[i] * s + (double)y[gmap[i]]);
}

__global__ void k_pair(const double* __restrict__ rh, const double* __restrict__ eh, const int32_t* __restrict__ gmap,
                       float* __restrict__ X, float* __restrict__ Y, double scale, int nf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    X[gmap[i]] = (float)(rh[i] * scale);
    Y[gmap[i]] = (float)(eh[i] * scale);
}

// d = (x + y - t) * mask; grad = 2 d * gscale; partial loss sums per block
__global__ void __launch_bounds__(kThreads) k_loss(const float* __restrict__ y, const float* __restrict__ x,
                                                   const float* __restrict__ t, const float* __restrict__ mask,
                                                   float* __restrict__ grad, float gscale, float* __restrict__ partial, int n3) {
    __shared__ float sh[kThreads / 32];
    float s = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += gridDim.x * blockDim.x) {
        const float dd = (x[i] + y[i] - t[i]) * mask[i];
        grad[i] = 2.f * dd * gscale;
        s = fmaf(dd, dd, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        float u = threadIdx.x < kThreads / 32 ? sh[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = u;
    }
}

__global__ void k_loss_final(const float* __restrict__ partial, float* out, int nblk) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        float s = 0.f;
        for (int b = 0; b < nblk; ++b) s += partial[b];
        out[0] += s;
    }
}

__global__ void k_adam(float* __restrict__ W, const float* __restrict__ G, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr_t, float b1, float b2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    W[i] -= lr_t * mi / (sqrtf(vi) + eps);
}


// ---------------------------------------------------------------------------
// Tensor-core inference path (tcgen05.mma.kind::f16, BF16 operands, FP32
// accumulation in TMEM).  Activations are channel-last BF16 grids [V][16].
// One CTA computes a tile of 8 (x) x 16 (y) x TCZ (z) voxels: the haloed
// block (10 x 18 x (TCZ+2) voxels) is staged by TMA in shared memory in the
// no-swizzle K-major canonical layout, channel group g (8 channels = 16 B)
// at g * TC_LBO, voxel (x, y, z) at z * TC_SZ + y * TC_SY + x * 16.  The
// A operand of halo plane h shifted by (dx, dy) is that block read from
// (h, 1 + dy, 1 + dx) with row stride TC_SY between 8-row groups: a shift is
// a descriptor offset, no data movement.  The three z taps are folded into
// N: for each (dx, dy) and halo plane h one M128 x N48 x K16 MMA multiplies
// A(h) by [W(dz=+1) | W(dz=0) | W(dz=-1)] into TMEM columns 16 h .. 16 h + 47,
// which hold the accumulators of output planes h-2, h-1, h (plane p lives at
// columns 16 (p + 2)).  9 (TCZ + 2) MMAs per tile instead of 27 TCZ.
constexpr int TCX = 8, TCY = 16, TCZ = 12;
constexpr int TC_HX = TCX + 2, TC_HY = TCY + 2, TC_HZ = TCZ + 2;
constexpr int TC_SY = TC_HX * 16;                 // 160 B
constexpr int TC_SZ = TC_HY * TC_SY;              // 2880 B
constexpr int TC_LBO = TC_HZ * TC_SZ;             // second channel group
constexpr int TC_A_BYTES = 2 * TC_LBO;
constexpr int TC_PAIRS = 9;                       // (dx, dy)
constexpr int TC_PAIR_BYTES = 48 * 16 * 2;        // N48 x K16 BF16 B operand
constexpr int TC_B_BYTES = TC_PAIRS * TC_PAIR_BYTES;
constexpr int TC_OFF_B = TC_A_BYTES;
constexpr int TC_OFF_BAR = TC_OFF_B + TC_B_BYTES;
constexpr int TC_SMEM = TC_OFF_BAR + 32;
constexpr int TC_THREADS = 128;
constexpr uint32_t TC_TMEM_COLS = 256;            // (TCZ + 4) planes x 16 columns, rounded up
constexpr long kTcWaitLimit = 4000000;
static_assert(TC_SY % 16 == 0 && TC_SZ % 16 == 0 && TC_LBO % 128 == 0, "descriptor strides / TMA destinations");
static_assert(TC_OFF_B % 128 == 0 && TC_OFF_BAR % 8 == 0, "alignment");
static_assert((TC_LBO >> 4) < (1 << 14) && (TC_SY >> 4) < (1 << 14), "descriptor fields");
static_assert((TCZ + 4) * 16 <= (int)TC_TMEM_COLS, "TMEM columns");
static_assert(TC_SMEM <= 227 * 1024, "shared memory");

// D = F32 (bits 4-5), A = B = BF16 (bits 7-9, 10-12), K-major, N >> 3, M >> 4
constexpr uint32_t kIdescBf16N48 = (1u << 4) | (1u << 7) | (1u << 10) | ((48u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t tc_smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// W fp32 [cout][cin][27] -> per-(dx, dy) B operand images: rows n = 16 blk + co
// with blk 0, 1, 2 <-> dz = +1, 0, -1; K = 16 input channels; K-major core
// matrices: (n/8)*256 + (k/8)*128 + (n%8)*16 + (k%8)*2 bytes.
__global__ void k_wprep(const float* __restrict__ W, __nv_bfloat16* __restrict__ out, int cin, int cout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;      // over 9 * 48 * 16
    if (i >= TC_PAIRS * 48 * 16) return;
    const int j = i / (48 * 16), n = (i / 16) % 48, k = i % 16;
    const int blk = n / 16, co = n % 16, dz = 1 - blk;
    const int t = (dz + 1) * 9 + j;                           // j = (dy+1)*3 + (dx+1)
    const float w = (co < cout && k < cin) ? W[(co * cin + k) * kNnTaps + t] : 0.f;
    const int off = j * (48 * 16) + (n / 8) * 128 + (k / 8) * 64 + (n % 8) * 8 + (k % 8);   // in bf16 units
    out[off] = __float2bfloat16_rn(w);
}

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS) k_conv_tc(const __grid_constant__ CUtensorMap tmap_in,
                                                         const __nv_bfloat16* __restrict__ wimg,
                                                         __nv_bfloat16* __restrict__ out_bf, float* __restrict__ out_f,
                                                         Dims d, int ntx, int nty, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char tsm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tsm + TC_OFF_BAR + 16);
    const uint32_t bar = tc_smem_u32(tsm + TC_OFF_BAR);            // MMA completion
    const uint32_t bar_tma = tc_smem_u32(tsm + TC_OFF_BAR + 8);    // halo arrival
    if (tc_smem_u32(tsm) & 127u) {                        // descriptors assume a 128 B aligned window
        if (tid == 0) atomicOr(status, 4);
        return;
    }
    const int tile = blockIdx.x;
    const int x0 = (tile % ntx) * TCX, y0 = ((tile / ntx) % nty) * TCY, z0 = (tile / (ntx * nty)) * TCZ;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(tc_smem_u32(tmem_slot)), "r"(TC_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(1) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar_tma), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // haloed block, one 8-channel group per copy; zero fill outside the lattice
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar_tma), "r"(TC_A_BYTES) : "memory");
#pragma unroll
        for (int g = 0; g < 2; ++g)
            asm volatile(
                "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
                :: "r"(tc_smem_u32(tsm + g * TC_LBO)), "l"(reinterpret_cast<uint64_t>(&tmap_in)), "r"(g * 8),
                   "r"(x0 - 1), "r"(y0 - 1), "r"(z0 - 1), "r"(bar_tma) : "memory");
    }
    // B operand images (27 taps)
    {
        const uint4* src = reinterpret_cast<const uint4*>(wimg);
        uint4* dst = reinterpret_cast<uint4*>(tsm + TC_OFF_B);
        for (int i = tid; i < TC_B_BYTES / 16; i += TC_THREADS) dst[i] = src[i];
    }
    const size_t plane = (size_t)d.nx * d.ny;
    __syncthreads();                                     // barriers initialised before anyone polls
    bool ok = false;
    for (long it = 0; it < kTcWaitLimit && !ok; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred q;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, q;\n\t}\n"
            : "=r"(done) : "r"(bar_tma), "r"(0u) : "memory");
        ok = done != 0;
    }
    ok = __syncthreads_and(ok);
    if (!ok) {                                          // halo never arrived: report, release TMEM, stop
        if (tid == 0) atomicOr(status, 2);
        if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(*tmem_slot), "r"(TC_TMEM_COLS) : "memory");
        return;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t abase = tc_smem_u32(tsm), bbase = tc_smem_u32(tsm + TC_OFF_B);
    const int nplanes = min(TCZ, d.nz - z0);
    // zero the accumulators (every MMA accumulates)
    {
        const uint32_t zr = 0u;
        for (int c = 0; c < (TCZ + 4) * 16; c += 16)
            asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};"
                         :: "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c), "r"(zr) : "memory");
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
        // halo planes h = 0 .. nplanes + 1 in residue classes mod 3, so that
        // consecutive MMAs write disjoint column ranges
        for (int j = 0; j < TC_PAIRS; ++j) {
            const int dx = j % 3 - 1, dy = j / 3 - 1;
            const uint64_t bdesc = tc_desc(bbase + j * TC_PAIR_BYTES, 128, 256);
            for (int r3 = 0; r3 < 3; ++r3) {
                for (int h = r3; h <= nplanes + 1; h += 3) {
                    const uint32_t aaddr = abase + h * TC_SZ + (1 + dy) * TC_SY + (1 + dx) * 16;
                    const uint64_t adesc = tc_desc(aaddr, TC_LBO, TC_SY);
                    asm volatile(
                        "{\n\t.reg .pred q;\n\t"
                        "setp.ne.b32 q, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, q;\n\t}\n"
                        :: "r"(tmem + (uint32_t)(h * 16)), "l"(adesc), "l"(bdesc), "r"(kIdescBf16N48), "r"(1u));
                }
            }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
    }
    // wait for the accumulators (bounded)
    ok = false;
    for (long it = 0; it < kTcWaitLimit && !ok; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred q;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, q;\n\t}\n"
            : "=r"(done) : "r"(bar), "r"(0u) : "memory");
        ok = done != 0;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) {
        if (tid == 0) atomicOr(status, 1);
    } else {
        const int m = tid;                                  // TMEM lane = tile row
        const int x = x0 + (m & 7), y = y0 + (m >> 3);
        for (int p = 0; p < nplanes; ++p) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((p + 2) * 16);
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                           "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int z = z0 + p;
            if (x < d.nx && y < d.ny) {
                const size_t v = (size_t)z * plane + (size_t)y * d.nx + x;
                if (MODE == 0) {
                    __align__(16) __nv_bfloat162 h[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        h[j] = __floats2bfloat162_rn(fmaxf(__uint_as_float(r[2 * j]), 0.f), fmaxf(__uint_as_float(r[2 * j + 1]), 0.f));
                    uint4* dst = reinterpret_cast<uint4*>(out_bf + v * 16);
                    dst[0] = *reinterpret_cast<uint4*>(&h[0]);
                    dst[1] = *reinterpret_cast<uint4*>(&h[4]);
                } else {
#pragma unroll
                    for (int c = 0; c < kNnOut; ++c) out_f[(size_t)c * d.V + v] = __uint_as_float(r[c]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
}

// features, channel-last BF16 [V][16], one thread per voxel (no pre-zeroing)
__global__ void k_feat_voxel_tc(const double* __restrict__ r, const double* __restrict__ sdinv,
                                const float* __restrict__ rho_grid, const int32_t* __restrict__ inv,
                                __nv_bfloat16* __restrict__ f, int V) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) h[c] = __float2bfloat16_rn(0.f);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int i = inv[(size_t)c * V + v];
        const float a = i >= 0 ? (float)(r[i] * sdinv[i]) : 0.f;
        h[c] = __float2bfloat16_rn(a);
        h[3 + c] = __float2bfloat16_rn(rho_grid[(size_t)c * V + v] * a);
    }
    uint4* dst = reinterpret_cast<uint4*>(f + (size_t)v * 16);
    dst[0] = *reinterpret_cast<uint4*>(&h[0]);
    dst[1] = *reinterpret_cast<uint4*>(&h[8]);
}

__global__ void k_feat_grid_tc(const float* __restrict__ x, const float* __restrict__ rho, __nv_bfloat16* __restrict__ f, int V) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) h[c] = __float2bfloat16_rn(0.f);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float a = x[(size_t)c * V + v];
        h[c] = __float2bfloat16_rn(a);
        h[3 + c] = __float2bfloat16_rn(rho[(size_t)c * V + v] * a);
    }
    uint4* dst = reinterpret_cast<uint4*>(f + (size_t)v * 16);
    dst[0] = *reinterpret_cast<uint4*>(&h[0]);
    dst[1] = *reinterpret_cast<uint4*>(&h[8]);
}

// TMA map of a channel-last BF16 grid [nz][ny][nx][16]: box = one 8-channel
// group of the haloed tile (8 x 10 x 18 x TC_HZ), zero fill outside.
int make_grid_map(const __nv_bfloat16* base, const Dims& d, CUtensorMap* map) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return SVL_ERR_CUDA;
        }
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const cuuint64_t dims[4] = {16, (cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)d.nz};
    const cuuint64_t strides[3] = {32, (cuuint64_t)d.nx * 32, (cuuint64_t)d.nx * d.ny * 32};
    const cuuint32_t box[4] = {8, TC_HX, TC_HY, TC_HZ};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(base), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return SVL_ERR_CUDA; }
    return SVL_OK;
}
static_assert(TC_HX * TC_HY * TC_HZ * 8 * 2 == TC_LBO, "one TMA box fills one channel-group block");

inline int nblocks(size_t n, int t = kThreads) { return (int)((n + t - 1) / t); }

// layer table: (cin, cout, offset into the weight vector)
struct Layer { int cin, cout, off; };
constexpr Layer kLayers[4] = {
    {kNnIn, kNnHid, 0},
    {kNnHid, kNnHid, kNnTaps * kNnIn * kNnHid},
    {kNnHid, kNnHid, kNnTaps * (kNnIn * kNnHid + kNnHid * kNnHid)},
    {kNnHid, kNnOut, kNnTaps * (kNnIn * kNnHid + 2 * kNnHid * kNnHid)},
};

}  // namespace

struct NnPrecond {
    Dims d{};
    int nf = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    int32_t* gmap = nullptr;
    double* sdinv = nullptr;
    float* rho = nullptr;      // [3][V]
    float* mask = nullptr;     // [3][V]
    float* W = nullptr;        // kNnWeights
    float* Wt = nullptr;       // flipped copy of one layer
    float* G = nullptr;        // gradient
    float *am = nullptr, *av = nullptr;
    float *feat = nullptr, *a0 = nullptr, *a1 = nullptr, *a2 = nullptr, *y = nullptr;   // forward
    float *g3 = nullptr, *gA = nullptr, *gB = nullptr;                                  // backward
    float* partial = nullptr;  // weight-gradient partials
    float* lpart = nullptr;    // loss partials
    float* lsum = nullptr;     // loss accumulator(s)
    std::vector<float*> X, Y;  // training pairs [3][V] each
    int nblk_wg = 0;
    // training on crops: window side (0 = the whole lattice) and window buffers
    int crop = 0;
    float *cx = nullptr, *ct = nullptr, *crho = nullptr, *cmask = nullptr;
    // tensor-core inference
    int use_tc = 1;
    bool tc_ready = false;
    __nv_bfloat16 *wimg = nullptr, *featc = nullptr, *actA = nullptr, *actB = nullptr;
    int* status = nullptr;
    int ntx = 0, nty = 0, ntz = 0;
    CUtensorMap map_feat{}, map_A{}, map_B{};
    int32_t* inv = nullptr;    // [3][V] free dof or -1

    template <typename T>
    int alloc(size_t n, T** p) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
            set_error("cudaMalloc of %zu bytes failed", n * sizeof(T));
            return SVL_ERR_NOMEM;
        }
        allocs.push_back(q);
        *p = (T*)q;
        return SVL_OK;
    }
    ~NnPrecond() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : allocs) cudaFree(p);
    }

    // forward of features already in `feat` on grid dd (the lattice or a
    // window of it); keeps activations
    int forward(const Dims& dd) {
        const int g = nblocks(dd.V);
        k_conv<kNnIn, kNnHid, true><<<g, kThreads, 0, stream>>>(feat, W + kLayers[0].off, a0, dd, nullptr);
        k_conv<kNnHid, kNnHid, true><<<g, kThreads, 0, stream>>>(a0, W + kLayers[1].off, a1, dd, nullptr);
        k_conv<kNnHid, kNnHid, true><<<g, kThreads, 0, stream>>>(a1, W + kLayers[2].off, a2, dd, nullptr);
        k_conv<kNnHid, kNnOut, false><<<g, kThreads, 0, stream>>>(a2, W + kLayers[3].off, y, dd, nullptr);
        NN_TRY(cudaGetLastError());
        return SVL_OK;
    }
    int forward() { return forward(d); }

    int prepare_tc() {
        for (int l = 0; l < 4; ++l)
            k_wprep<<<nblocks(TC_PAIRS * 48 * 16), kThreads, 0, stream>>>(W + kLayers[l].off, wimg + (size_t)l * TC_PAIRS * 48 * 16,
                                                                          kLayers[l].cin, kLayers[l].cout);
        NN_TRY(cudaGetLastError());
        tc_ready = true;
        return SVL_OK;
    }

    // tensor-core forward of the BF16 features in `featc`; output y (FP32 [3][V])
    // tensor-core forward of the BF16 features in `featc`; output y (FP32 [3][V])
    int forward_tc() {
        if (!tc_ready) if (int st = prepare_tc()) return st;
        const int nt = ntx * nty * ntz;
        const size_t lw = (size_t)TC_PAIRS * 48 * 16;
        k_conv_tc<0><<<nt, TC_THREADS, TC_SMEM, stream>>>(map_feat, wimg, actA, nullptr, d, ntx, nty, status);
        k_conv_tc<0><<<nt, TC_THREADS, TC_SMEM, stream>>>(map_A, wimg + lw, actB, nullptr, d, ntx, nty, status);
        k_conv_tc<0><<<nt, TC_THREADS, TC_SMEM, stream>>>(map_B, wimg + 2 * lw, actA, nullptr, d, ntx, nty, status);
        k_conv_tc<1><<<nt, TC_THREADS, TC_SMEM, stream>>>(map_A, wimg + 3 * lw, nullptr, y, d, ntx, nty, status);
        NN_TRY(cudaGetLastError());
        return SVL_OK;
    }

    template <int CIN, int COUT>
    int wgrad(const float* gout, const float* ain, int layer, const Dims& dd) {
        const int nb = (dd.V + kWgChunk - 1) / kWgChunk;
        dim3 grid(nb, kNnTaps);
        k_wgrad<CIN, COUT><<<grid, kThreads, 0, stream>>>(gout, ain, partial, dd);
        const int n = CIN * COUT * kNnTaps;
        k_wgrad_reduce<<<nblocks(n), kThreads, 0, stream>>>(partial, G + kLayers[layer].off, CIN, COUT, nb);
        NN_TRY(cudaGetLastError());
        return SVL_OK;
    }

    // data gradient through layer `layer` (cout -> cin), gated by the layer input's relu
    template <int CIN, int COUT>
    int dgrad(const float* gout, float* gin, const float* gate, int layer, const Dims& dd) {
        const int n = CIN * COUT * kNnTaps;
        k_flip<<<nblocks(n), kThreads, 0, stream>>>(W + kLayers[layer].off, Wt, CIN, COUT);
        k_conv<COUT, CIN, false><<<nblocks(dd.V), kThreads, 0, stream>>>(gout, Wt, gin, dd, gate);
        NN_TRY(cudaGetLastError());
        return SVL_OK;
    }

    // features of one pair on grid dd (rho and mask of that grid), forward,
    // loss into lslot, gradient accumulated into G
    int sample(const float* x, const float* t, float gscale, float* lslot, const Dims& dd, const float* rg,
               const float* mg) {
        const int n3 = 3 * dd.V;
        k_feat_grid<<<nblocks(n3), kThreads, 0, stream>>>(x, rg, feat, n3);
        if (int st = forward(dd)) return st;
        k_loss<<<kRedBlocks, kThreads, 0, stream>>>(y, x, t, mg, g3, gscale, lpart, n3);
        k_loss_final<<<1, 32, 0, stream>>>(lpart, lslot, kRedBlocks);
        if (int st = wgrad<kNnHid, kNnOut>(g3, a2, 3, dd)) return st;
        if (int st = dgrad<kNnHid, kNnOut>(g3, gA, a2, 3, dd)) return st;
        if (int st = wgrad<kNnHid, kNnHid>(gA, a1, 2, dd)) return st;
        if (int st = dgrad<kNnHid, kNnHid>(gA, gB, a1, 2, dd)) return st;
        if (int st = wgrad<kNnHid, kNnHid>(gB, a0, 1, dd)) return st;
        if (int st = dgrad<kNnHid, kNnHid>(gB, gA, a0, 1, dd)) return st;
        if (int st = wgrad<kNnIn, kNnHid>(gA, feat, 0, dd)) return st;
        return SVL_OK;
    }
    int sample(const float* x, const float* t, float gscale, float* lslot) {
        return sample(x, t, gscale, lslot, d, rho, mask);
    }
};

int nn_create(int nx, int ny, int nz, const std::vector<int32_t>& gmap, const std::vector<double>& sdinv,
              const std::vector<double>& rho, cudaStream_t stream, NnPrecond** out) {
    *out = nullptr;
    NnPrecond* nn = new NnPrecond();
    auto fail = [&](int st) { delete nn; return st; };
    nn->d = {nx, ny, nz, nx * ny * nz};
    nn->nf = (int)gmap.size();
    nn->stream = stream;
    const size_t V = (size_t)nn->d.V;
    int st;
    if ((st = nn->alloc(gmap.size(), &nn->gmap)) || (st = nn->alloc(sdinv.size(), &nn->sdinv)) ||
        (st = nn->alloc(3 * V, &nn->rho)) || (st = nn->alloc(3 * V, &nn->mask)) ||
        (st = nn->alloc(kNnWeights, &nn->W)) || (st = nn->alloc(kNnHid * kNnHid * kNnTaps, &nn->Wt)) ||
        (st = nn->alloc(kNnWeights, &nn->G)) || (st = nn->alloc(kNnWeights, &nn->am)) ||
        (st = nn->alloc(kNnWeights, &nn->av)) || (st = nn->alloc(kNnIn * V, &nn->feat)) ||
        (st = nn->alloc(kNnHid * V, &nn->a0)) || (st = nn->alloc(kNnHid * V, &nn->a1)) ||
        (st = nn->alloc(kNnHid * V, &nn->a2)) || (st = nn->alloc(kNnOut * V, &nn->y)) ||
        (st = nn->alloc(kNnOut * V, &nn->g3)) || (st = nn->alloc(kNnHid * V, &nn->gA)) ||
        (st = nn->alloc(kNnHid * V, &nn->gB)) || (st = nn->alloc(kRedBlocks, &nn->lpart)) ||
        (st = nn->alloc(1 << 16, &nn->lsum)))
        return fail(st);
    nn->nblk_wg = (int)((V + kWgChunk - 1) / kWgChunk);
    nn->ntx = (nx + TCX - 1) / TCX;
    nn->nty = (ny + TCY - 1) / TCY;
    nn->ntz = (nz + TCZ - 1) / TCZ;
    if ((st = nn->alloc((size_t)4 * TC_PAIRS * 48 * 16, &nn->wimg)) || (st = nn->alloc(16 * V, &nn->featc)) ||
        (st = nn->alloc(16 * V, &nn->actA)) || (st = nn->alloc(16 * V, &nn->actB)) || (st = nn->alloc(4, &nn->status)))
        return fail(st);
    NN_TRY(cudaMemsetAsync(nn->status, 0, sizeof(int), stream));
    {
        std::vector<int32_t> inv(3 * V, -1);
        for (size_t f = 0; f < gmap.size(); ++f) inv[gmap[f]] = (int32_t)f;
        if ((st = nn->alloc(3 * V, &nn->inv))) return fail(st);
        NN_TRY(cudaMemcpyAsync(nn->inv, inv.data(), inv.size() * 4, cudaMemcpyHostToDevice, stream));
        NN_TRY(cudaStreamSynchronize(stream));
    }
    if ((st = make_grid_map(nn->featc, nn->d, &nn->map_feat)) || (st = make_grid_map(nn->actA, nn->d, &nn->map_A)) ||
        (st = make_grid_map(nn->actB, nn->d, &nn->map_B)))
        return fail(st);
    {
        static bool attr_set = false;
        if (!attr_set) {
            NN_TRY(cudaFuncSetAttribute(k_conv_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
            NN_TRY(cudaFuncSetAttribute(k_conv_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
            attr_set = true;
        }
    }
    if ((st = nn->alloc((size_t)nn->nblk_wg * kNnTaps * kNnHid * kNnHid, &nn->partial))) return fail(st);
    // host-side grids: rho and mask on the lattice
    std::vector<float> rg(3 * V, 0.f), mg(3 * V, 0.f);
    for (size_t f = 0; f < gmap.size(); ++f) {
        rg[gmap[f]] = (float)rho[f];
        mg[gmap[f]] = 1.f;
    }
    // He-style initialisation, small last layer (the net starts as plain Jacobi)
    std::vector<float> w(kNnWeights);
    uint64_t s = 0x9E3779B97F4A7C15ull;
    auto unif = [&]() {
        s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
        return (double)((s * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < 4; ++l) {
        const int n = kLayers[l].cin * kLayers[l].cout * kNnTaps;
        const double a = std::sqrt(6.0 / (kLayers[l].cin * kNnTaps)) * (l == 3 ? 0.1 : 1.0);
        for (int i = 0; i < n; ++i) w[kLayers[l].off + i] = (float)((2.0 * unif() - 1.0) * a);
    }
    NN_TRY(cudaMemcpyAsync(nn->gmap, gmap.data(), gmap.size() * 4, cudaMemcpyHostToDevice, stream));
    NN_TRY(cudaMemcpyAsync(nn->sdinv, sdinv.data(), sdinv.size() * 8, cudaMemcpyHostToDevice, stream));
    NN_TRY(cudaMemcpyAsync(nn->rho, rg.data(), rg.size() * 4, cudaMemcpyHostToDevice, stream));
    NN_TRY(cudaMemcpyAsync(nn->mask, mg.data(), mg.size() * 4, cudaMemcpyHostToDevice, stream));
    NN_TRY(cudaMemcpyAsync(nn->W, w.data(), w.size() * 4, cudaMemcpyHostToDevice, stream));
    NN_TRY(cudaStreamSynchronize(stream));
    *out = nn;
    return SVL_OK;
}

void nn_destroy(NnPrecond* nn) { delete nn; }

int nn_apply(NnPrecond* nn, const double* r, double* z) {
    const int n3 = 3 * nn->d.V;
    if (nn->use_tc) {
        k_feat_voxel_tc<<<nblocks(nn->d.V), kThreads, 0, nn->stream>>>(r, nn->sdinv, nn->rho, nn->inv, nn->featc, nn->d.V);
        if (int st = nn->forward_tc()) return st;
    } else {
        NN_TRY(cudaMemsetAsync(nn->feat, 0, sizeof(float) * kNnIn * (size_t)nn->d.V, nn->stream));
        k_feat_free<<<nblocks(nn->nf), kThreads, 0, nn->stream>>>(r, nn->sdinv, nn->rho, nn->gmap, nn->feat, nn->nf, n3);
        if (int st = nn->forward()) return st;
    }
    k_out_free<<<nblocks(nn->nf), kThreads, 0, nn->stream>>>(nn->y, r, nn->sdinv, nn->gmap, z, nn->nf);
    NN_TRY(cudaGetLastError());
    return SVL_OK;
}

int nn_record_pair(NnPrecond* nn, const double* rhat, const double* ehat, double scale) {
    float *X = nullptr, *Y = nullptr;
    const size_t n3 = 3 * (size_t)nn->d.V;
    if (int st = nn->alloc(n3, &X)) return st;
    if (int st = nn->alloc(n3, &Y)) return st;
    NN_TRY(cudaMemsetAsync(X, 0, n3 * 4, nn->stream));
    NN_TRY(cudaMemsetAsync(Y, 0, n3 * 4, nn->stream));
    k_pair<<<nblocks(nn->nf), kThreads, 0, nn->stream>>>(rhat, ehat, nn->gmap, X, Y, scale, nn->nf);
    NN_TRY(cudaGetLastError());
    nn->X.push_back(X);
    nn->Y.push_back(Y);
    return SVL_OK;
}

int nn_num_pairs(const NnPrecond* nn) { return (int)nn->X.size(); }

int nn_train_segment(NnPrecond* nn, int it_begin, int it_end, int iters, int batch, float lr, uint64_t seed, float* loss) {
    const int np = (int)nn->X.size();
    if (np == 0 || iters <= 0 || batch <= 0 || it_begin < 0 || it_end > iters || it_begin >= it_end) {
        set_error("nothing to train on");
        return SVL_ERR_INVALID;
    }
    if (iters > (1 << 16)) { set_error("at most 65536 training iterations"); return SVL_ERR_INVALID; }
    if (it_begin == 0) {
        NN_TRY(cudaMemsetAsync(nn->am, 0, sizeof(float) * kNnWeights, nn->stream));
        NN_TRY(cudaMemsetAsync(nn->av, 0, sizeof(float) * kNnWeights, nn->stream));
    }
    NN_TRY(cudaMemsetAsync(nn->lsum + it_begin, 0, sizeof(float) * (it_end - it_begin), nn->stream));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int it = it_begin; it < it_end; ++it) {
        NN_TRY(cudaMemsetAsync(nn->G, 0, sizeof(float) * kNnWeights, nn->stream));
        for (int b = 0; b < batch; ++b) {
            // pair index from a counter-based hash of (seed, iteration, slot)
            uint64_t h = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(it * 131 + b + 1));
            h ^= h >> 31; h *= 0xBF58476D1CE4E5B9ull; h ^= h >> 29;
            const int p = (int)(h % (uint64_t)np);
            if (nn->crop > 0) {
                // a window of side crop at an offset drawn from the same hash
                const Dims& f = nn->d;
                Dims cr{std::min(nn->crop, f.nx), std::min(nn->crop, f.ny), std::min(nn->crop, f.nz), 0};
                cr.V = cr.nx * cr.ny * cr.nz;
                uint64_t h2 = h * 0x94D049BB133111EBull;
                h2 ^= h2 >> 31;
                const int ox = (int)(h2 % (uint64_t)(f.nx - cr.nx + 1));
                const int oy = (int)((h2 >> 20) % (uint64_t)(f.ny - cr.ny + 1));
                const int oz = (int)((h2 >> 40) % (uint64_t)(f.nz - cr.nz + 1));
                const int g3 = nblocks(3 * cr.V);
                k_crop<<<g3, kThreads, 0, nn->stream>>>(nn->X[p], nn->cx, f, cr, ox, oy, oz);
                k_crop<<<g3, kThreads, 0, nn->stream>>>(nn->Y[p], nn->ct, f, cr, ox, oy, oz);
                k_crop<<<g3, kThreads, 0, nn->stream>>>(nn->rho, nn->crho, f, cr, ox, oy, oz);
                k_crop_mask<<<g3, kThreads, 0, nn->stream>>>(nn->mask, nn->cmask, f, cr, ox, oy, oz, 4);
                if (int st = nn->sample(nn->cx, nn->ct, 1.f / batch, nn->lsum + it, cr, nn->crho, nn->cmask)) return st;
                continue;
            }
            if (int st = nn->sample(nn->X[p], nn->Y[p], 1.f / batch, nn->lsum + it)) return st;
        }
        const float frac = (float)it / iters;
        const float lr_it = lr * (frac < 0.6f ? 1.f : (frac < 0.85f ? 0.25f : 0.05f));
        const double c1 = 1.0 - std::pow((double)b1, it + 1), c2 = 1.0 - std::pow((double)b2, it + 1);
        const float lr_t = (float)(lr_it * std::sqrt(c2) / c1);
        k_adam<<<nblocks(kNnWeights), kThreads, 0, nn->stream>>>(nn->W, nn->G, nn->am, nn->av, kNnWeights, lr_t, b1, b2, eps);
        NN_TRY(cudaGetLastError());
    }
    nn->tc_ready = false;
    const int n = it_end - it_begin;
    std::vector<float> lh(n);
    NN_TRY(cudaMemcpyAsync(lh.data(), nn->lsum + it_begin, sizeof(float) * n, cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    const int tail = std::max(1, n / 10);
    double acc = 0.0;
    for (int i = n - tail; i < n; ++i) acc += lh[i];
    if (loss) *loss = (float)(acc / tail / batch);
    if (!std::isfinite(acc)) { set_error("training diverged"); return SVL_ERR_NONFINITE; }
    return SVL_OK;
}

int nn_set_crop(NnPrecond* nn, int crop) {
    if (crop < 0) { set_error("crop must be >= 0"); return SVL_ERR_INVALID; }
    if (crop > 0 && crop < 9) { set_error("crop windows need at least 9 voxels a side"); return SVL_ERR_INVALID; }
    if (crop > 0 && !nn->cx) {
        const size_t n = (size_t)3 * std::min(crop, nn->d.nx) * std::min(crop, nn->d.ny) * std::min(crop, nn->d.nz);
        int st;
        if ((st = nn->alloc(n, &nn->cx)) || (st = nn->alloc(n, &nn->ct)) || (st = nn->alloc(n, &nn->crho)) ||
            (st = nn->alloc(n, &nn->cmask)))
            return st;
    } else if (crop > nn->crop && nn->cx && nn->crop > 0) {
        set_error("the crop size is fixed by the first training with crops"); return SVL_ERR_INVALID;
    }
    nn->crop = crop;
    return SVL_OK;
}

int nn_train(NnPrecond* nn, int iters, int batch, float lr, uint64_t seed, float* loss) {
    return nn_train_segment(nn, 0, iters, iters, batch, lr, seed, loss);
}

int nn_set_weights(NnPrecond* nn, const float* w) {
    nn->tc_ready = false;
    NN_TRY(cudaMemcpyAsync(nn->W, w, sizeof(float) * kNnWeights, cudaMemcpyHostToDevice, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    return SVL_OK;
}

int nn_get_weights(NnPrecond* nn, float* w) {
    NN_TRY(cudaMemcpyAsync(w, nn->W, sizeof(float) * kNnWeights, cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    return SVL_OK;
}

int nn_loss_grad_host(NnPrecond* nn, const float* x, const float* t, float* loss, float* grad) {
    const size_t n3 = 3 * (size_t)nn->d.V;
    float *X = nullptr, *T = nullptr;
    if (int st = nn->alloc(n3, &X)) return st;
    if (int st = nn->alloc(n3, &T)) return st;
    NN_TRY(cudaMemcpyAsync(X, x, n3 * 4, cudaMemcpyHostToDevice, nn->stream));
    NN_TRY(cudaMemcpyAsync(T, t, n3 * 4, cudaMemcpyHostToDevice, nn->stream));
    NN_TRY(cudaMemsetAsync(nn->G, 0, sizeof(float) * kNnWeights, nn->stream));
    NN_TRY(cudaMemsetAsync(nn->lsum, 0, sizeof(float), nn->stream));
    if (int st = nn->sample(X, T, 1.f, nn->lsum)) return st;
    NN_TRY(cudaMemcpyAsync(grad, nn->G, sizeof(float) * kNnWeights, cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaMemcpyAsync(loss, nn->lsum, sizeof(float), cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    return SVL_OK;
}

int nn_forward_host(NnPrecond* nn, const float* x, float* y, int path) {
    const size_t n3 = 3 * (size_t)nn->d.V;
    float* X = nullptr;
    if (int st = nn->alloc(n3, &X)) return st;
    NN_TRY(cudaMemcpyAsync(X, x, n3 * 4, cudaMemcpyHostToDevice, nn->stream));
    if (path == 1) {
        k_feat_grid_tc<<<nblocks(nn->d.V), kThreads, 0, nn->stream>>>(X, nn->rho, nn->featc, nn->d.V);
        if (int st = nn->forward_tc()) return st;
    } else {
        k_feat_grid<<<nblocks(n3), kThreads, 0, nn->stream>>>(X, nn->rho, nn->feat, (int)n3);
        if (int st = nn->forward()) return st;
    }
    NN_TRY(cudaMemcpyAsync(y, nn->y, n3 * 4, cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    return nn_status(nn);
}

int nn_status(NnPrecond* nn) {
    int h = 0;
    NN_TRY(cudaMemcpyAsync(&h, nn->status, sizeof(int), cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    if (h) {
        set_error("tensor-core convolution reported status %d (1 = accumulator wait gave up, 4 = misaligned shared memory)", h);
        return SVL_ERR_CUDA;
    }
    return SVL_OK;
}

void nn_set_path(NnPrecond* nn, int path) { nn->use_tc = path == 1; }

int nn_get_grids(NnPrecond* nn, float* rho, float* mask) {
    const size_t n3 = 3 * (size_t)nn->d.V;
    if (rho) NN_TRY(cudaMemcpyAsync(rho, nn->rho, n3 * 4, cudaMemcpyDeviceToHost, nn->stream));
    if (mask) NN_TRY(cudaMemcpyAsync(mask, nn->mask, n3 * 4, cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    return SVL_OK;
}

}  // namespace svl
