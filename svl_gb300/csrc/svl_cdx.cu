// Mixed-precision batched central difference on uniform lin3DHexa8 grids.
//
// One fused kernel per step (k_cdx_step).  Each CTA owns a TX x TY x TZ block
// of nodes of one instance and
//   1. stages the (TX+2) x (TY+2) x (TZ+2) halo of FP64 displacements and the
//      lambda/mu of the (TX+1)(TY+1)(TZ+1) elements touching its nodes in
//      shared memory;
//   2. computes those elements' internal forces as a tcgen05 GEMM, 128
//      elements per MMA tile:  D[128 x 48] = U_e[128 x 24] . [K_lambda; K_mu]^T,
//      with TF32 hi/lo operands (lo.hi + hi.lo + hi.hi accumulated in one FP32
//      TMEM accumulator; eight accumulator slots so the MMAs of the next tile
//      run while the update of this one is in progress), then
//      F_e = lambda_e D[:, 0:24] + mu_e D[:, 24:48];
//   3. gathers the eight element contributions of every owned node in the
//      reference's element-tag order (no atomics) and updates
//      u_{n+1} = u_n + (u_n - u_{n-1}) + (dt^2/m)(f_ext - f_int)
//      (CentralDifference.cpp:138-148 with the diagonal solve, for lumped
//      mass without damping).
// The displacement state is kept as a compensated pair of FP32 numbers
// (u = hi + lo, about 48 significant bits) updated with error-free TwoSum
// transformations, so the hot loop issues no FP64 instruction: on GB300 the
// FP64 pipe (about 1.2 TFLOP/s) cannot keep up with even an FP64 axpy over
// the state at HBM speed.  Host-side reads and writes convert to and from FP64.
// Element-local dof order and node order follow lin3DHexa8.cpp:756-853.
// A small k_cdx_loads kernel adds (dt^2/m) f_ext for the loaded dofs.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

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

constexpr int align_up(int x, int a) { return (x + a - 1) / a * a; }

// Node tile owned by one CTA per pass and derived sizes.
constexpr int TX = 8, TY = 8, TZ = 8;
constexpr int HY = TY + 2, HZ = TZ + 2;                       // halo nodes in y, z (x: RAWX floats)
constexpr int EX = TX + 1, EY = TY + 1, EZ = TZ + 1;          // elements touching the tile
constexpr int NEL = EX * EY * EZ;                             // 729
constexpr int NMT = (NEL + 127) / 128;                        // 6 MMA tiles of 128 elements
constexpr int NTHREADS = 512;                                 // 16 warps
constexpr int NBUILD = 256;                                   // warps 0-7 build operands
constexpr int ISSUE_WARP = 8;                                 // warp 8 issues the MMAs
constexpr int UPD_WARP0 = 9;                                  // warps 9-15 gather and update
constexpr int NUPD = NTHREADS - UPD_WARP0 * 32;               // 224 threads
constexpr int EPI_WARP0 = 12;                                 // warps 12-15 also drain TMEM
constexpr int NEPI = 128;
constexpr int RAWX = 40;                                      // TMA box: floats per halo row
constexpr int RAW_SHIFT = 3;                                  // halo row starts 3 nodes left of x0-1
constexpr int RAW_BYTES = RAWX * HY * HZ * 4;                 // 16000 B
constexpr int LMX = 16;                                       // TMA box: lambda/mu floats per row
constexpr int LM_SHIFT = 3;                                   // element row starts 3 left of x0-1
constexpr int LM_BYTES = LMX * EY * EZ * 4;                   // 5184 B each
constexpr int OWN_BYTES = TX * 3 * TY * TZ * 4;               // 6144 B per owned-node array
constexpr int HALO_TX_BYTES = RAW_BYTES + 2 * LM_BYTES;       // halo + lambda + mu per tile
constexpr int OWN_TX_BYTES = 4 * OWN_BYTES;                   // owned-node state per tile
constexpr int FSTRIDE = 25;                                   // padded row of element forces

// Canonical no-swizzle K-major operand layout: 8-row x 16-byte core matrices;
// element (r, k) at (r/8)*SBO + (k/4)*LBO + (r%8)*16 + (k%4)*4 bytes.
constexpr int KDIM = 24;                                      // element dofs
constexpr int LBO = 128;                                      // next core matrix along K
constexpr int SBO = (KDIM / 4) * 128;                         // next 8 rows: 768 B
constexpr int A_BYTES = (128 / 8) * SBO;                      // 12288 B per operand
constexpr int B_ROWS = 96;                                    // [K_stack hi (48 rows); K_stack lo (48 rows)]
constexpr int B_BYTES = (B_ROWS / 8) * SBO;                   // 9216 B

constexpr int OFF_B = 0;
constexpr int OFF_A = align_up(OFF_B + B_BYTES, 1024);       // [2 buffers][hi, lo]
constexpr int A_STRIDE = 2 * A_BYTES;
constexpr int OFF_TT = OFF_A + 2 * A_STRIDE;                   // [2 buffers] halo of u_n (high part), lambda, mu
constexpr int TT_LAM = align_up(RAW_BYTES, 128);
constexpr int TT_MU = align_up(TT_LAM + LM_BYTES, 128);
constexpr int TT_STRIDE = align_up(TT_MU + LM_BYTES, 1024);
constexpr int OFF_OWN = OFF_TT + 2 * TT_STRIDE;                  // owned: u_n low, u_{n-1} hi/lo, dt^2/m
constexpr int OWN_ULC = 0, OWN_UHP = OWN_BYTES, OWN_ULP = 2 * OWN_BYTES, OWN_CD = 3 * OWN_BYTES;
constexpr int OFF_F = align_up(OFF_OWN + 4 * OWN_BYTES, 128);    // element forces
constexpr int OFF_BAR = align_up(OFF_F + NEL * FSTRIDE * 4, 16);
constexpr int NDB = 8;                                        // accumulator slots in TMEM (a tile's 6 M-tiles fit)
constexpr int NBAR = 7 + 2 * NDB;                             // tma[2] a_full[2] a_empty[2] own d_full[NDB] d_empty[NDB]
constexpr int OFF_TMEM = OFF_BAR + NBAR * 8;
constexpr int SMEM_BYTES = OFF_TMEM + 16;
static_assert(OFF_A % 1024 == 0 && A_STRIDE % 1024 == 0, "MMA operands on 1 KB boundaries");
static_assert(OFF_TT % 1024 == 0 && TT_STRIDE % 1024 == 0 && TT_LAM % 128 == 0 && TT_MU % 128 == 0 &&
              OFF_OWN % 128 == 0 && OWN_BYTES % 128 == 0, "TMA destinations");
static_assert(OFF_F % 16 == 0 && OFF_BAR % 8 == 0 && OFF_TMEM % 4 == 0, "alignment");
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory budget");
static_assert(TX * TY * TZ <= 3 * NUPD, "three owned nodes per update thread at most");

constexpr uint32_t ACC_COLS = 64;       // 48 accumulator columns per slot
constexpr uint32_t TMEM_COLS = NDB * ACC_COLS;
constexpr uint32_t B_LO_OFF = (48 / 8) * SBO;   // K lo rows of the B image
constexpr long kWaitLimit = 4000000;    // bounded mbarrier wait

// Instruction descriptors for tcgen05.mma.kind::tf32: D = F32 (bits 4-5),
// A = B = TF32 (bits 7-9, 10-12), both K-major, N >> 3 (bits 17-22),
// M >> 4 (bits 24-28).
constexpr uint32_t idesc_tf32(uint32_t m, uint32_t n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}
constexpr uint32_t kIdescN48 = idesc_tf32(128, 48);

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

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
        :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(bar) : "memory");
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

// TMA: 4D tiled load, completion counted on `bar` (expect_tx set by the caller).
__device__ __forceinline__ void tma_load4(const CUtensorMap* tmap, uint32_t dst, uint32_t bar, int x, int y, int z, int w) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        :: "r"(dst), "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar) : "memory");
}

template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float* v);
template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

struct CdxView {
    int nx, ny, nz, ninst;
    int pitch;                           // floats per padded x-row of the state arrays
    int ntx, nty, ntz, ntiles;
    float* uh_prev;                      // u_{n-1} (read through TMA), u_{n+1} written here
    float* ul_prev;
    const float* __restrict__ cdof;      // [inst][z][y][pitch]  dt^2/m, 0 on restrained dofs
    const float* __restrict__ bop;       // [B_ROWS x 24] hi then lo operand image
    // external loads grouped by tile, then by dof
    const int* __restrict__ tl_ptr;      // [ntiles+1] into the unique-dof arrays
    const long long* __restrict__ ld_dof;// padded index of the dof
    const int* __restrict__ ld_ptr;      // [nld+1] into ser/coef
    const int* __restrict__ ld_ser;
    const double* __restrict__ ld_coef;
    const int* __restrict__ s_ptr;
    const double* __restrict__ s_val;
    int k;                               // step index
    int* status;
};

// Error-free transformations on FP32 (Knuth TwoSum, Dekker FastTwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
// (ah + al) + (bh + bl) as a normalised pair.
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float& rh, float& rl) {
    float s, e;
    two_sum(ah, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, bl));
    fast_two_sum(s, e, rh, rl);
}

// AND of `v` over the warps 9-15 group, on named barrier 2 (also a memory barrier for the group).
__device__ __forceinline__ bool group_and(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, 2, %2, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r) : "r"((uint32_t)v), "r"(NUPD) : "memory");
    return r != 0;
}

struct TileOrigin { int inst, x0, y0, z0; };
__device__ __forceinline__ TileOrigin tile_origin(const CdxView& v, int tile) {
    TileOrigin o;
    int r = tile;
    const int tx = r % v.ntx; r /= v.ntx;
    const int ty = r % v.nty; r /= v.nty;
    const int tz = r % v.ntz;
    o.inst = r / v.ntz;
    o.x0 = tx * TX; o.y0 = ty * TY; o.z0 = tz * TZ;
    return o;
}

__global__ void __launch_bounds__(NTHREADS, 1)
k_cdx_step(const __grid_constant__ CUtensorMap tmap_u, const __grid_constant__ CUtensorMap tmap_lam,
           const __grid_constant__ CUtensorMap tmap_mu, const __grid_constant__ CUtensorMap tmap_ulc,
           const __grid_constant__ CUtensorMap tmap_uhp, const __grid_constant__ CUtensorMap tmap_ulp,
           const __grid_constant__ CUtensorMap tmap_cd, CdxView v) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int nxn = v.nx + 1, nyn = v.ny + 1, nzn = v.nz + 1;
    float* sF = reinterpret_cast<float*>(smem + OFF_F);     // element forces of the tile
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + OFF_TMEM);
    // barrier addresses are computed (no small arrays indexed at run time: those live in local memory)
    const uint32_t bar0 = smem_u32(bars);
#define B_TMA(b) (bar0 + 8u * (uint32_t)(b))
#define B_AFULL(b) (bar0 + 16u + 8u * (uint32_t)(b))
#define B_AEMPTY(b) (bar0 + 32u + 8u * (uint32_t)(b))
#define B_DFULL(b) (bar0 + 56u + 8u * (uint32_t)(b))
#define B_DEMPTY(b) (bar0 + 56u + 8u * NDB + 8u * (uint32_t)(b))
    const uint32_t b_own = bar0 + 48u;
// phase bits of two-slot barriers packed in one word
#define PH(w, b) (((w) >> (b)) & 1u)
#define FLIP(w, b) ((w) ^= (1u << (b)))
    // TMA destinations and MMA operands assume a 1 KB aligned dynamic window
    if (smem_u32(smem) & 1023u) {
        if (tid == 0) atomicOr(v.status, 2);
        return;
    }

    // -- once per CTA: TMEM, barriers, B operand ----------------------------
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(tmem_slot)), "r"(TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            mbar_init(B_TMA(b), 1);
            mbar_init(B_AFULL(b), NBUILD);
            mbar_init(B_AEMPTY(b), 1);
        }
        for (int b = 0; b < NDB; ++b) {
            mbar_init(B_DFULL(b), 1);
            mbar_init(B_DEMPTY(b), NEPI);
        }
        mbar_init(b_own, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    {
        const float4* src = reinterpret_cast<const float4*>(v.bop);
        float4* dst = reinterpret_cast<float4*>(smem + OFF_B);
        for (int i = tid; i < B_BYTES / 16; i += NTHREADS) dst[i] = src[i];
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    auto issue_tile = [&](int tile, int buf) {
        const TileOrigin o = tile_origin(v, tile);
        const uint32_t dst = smem_u32(smem + OFF_TT + buf * TT_STRIDE);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(B_TMA(buf)), "r"(HALO_TX_BYTES) : "memory");
        tma_load4(&tmap_u, dst, B_TMA(buf), (o.x0 - 1 - RAW_SHIFT) * 3, o.y0 - 1, o.z0 - 1, o.inst);
        tma_load4(&tmap_lam, dst + TT_LAM, B_TMA(buf), o.x0 - 1 - LM_SHIFT, o.y0 - 1, o.z0 - 1, o.inst);
        tma_load4(&tmap_mu, dst + TT_MU, B_TMA(buf), o.x0 - 1 - LM_SHIFT, o.y0 - 1, o.z0 - 1, o.inst);
    };
    auto issue_owned = [&](int tile) {
        const TileOrigin o = tile_origin(v, tile);
        const uint32_t dst = smem_u32(smem + OFF_OWN);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(b_own), "r"(OWN_TX_BYTES) : "memory");
        tma_load4(&tmap_ulc, dst + OWN_ULC, b_own, o.x0 * 3, o.y0, o.z0, o.inst);
        tma_load4(&tmap_uhp, dst + OWN_UHP, b_own, o.x0 * 3, o.y0, o.z0, o.inst);
        tma_load4(&tmap_ulp, dst + OWN_ULP, b_own, o.x0 * 3, o.y0, o.z0, o.inst);
        tma_load4(&tmap_cd, dst + OWN_CD, b_own, o.x0 * 3, o.y0, o.z0, o.inst);
    };
    const int ntile_cta = v.ntiles > (int)blockIdx.x ? (v.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    bool ok = true;

    if (warp < NBUILD / 32) {
        // ===== builders: A operand rows (element x 24 dofs), TF32 hi / lo =====
        uint32_t ph_tma = 0u, ph_aempty = 3u;
        const int h = tid >> 7, m = tid & 127;
        for (int it = 0, mt = 0; it < ntile_cta && ok; ++it) {
            const int buf = it & 1;
            ok = mbar_wait(B_TMA(buf), PH(ph_tma, buf));
            FLIP(ph_tma, buf);
            const float* raw = reinterpret_cast<const float*>(smem + OFF_TT + buf * TT_STRIDE);
            for (int t = 0; t < NMT && ok; ++t, ++mt) {
                const int b = mt & 1;
                ok = mbar_wait(B_AEMPTY(b), PH(ph_aempty, b));
                FLIP(ph_aempty, b);
                if (!ok) break;
                const int le = t * 128 + m;
                float hv[12], lv[12];
                if (le < NEL) {
                    const int lx = le % EX, ly = (le / EX) % EY, lz = le / (EX * EY);
                    // nodes n1..n4 (h = 0) or n5..n8 (h = 1) of the element, in the raw halo rows
                    const int r0 = (lz + h) * HY + ly;
                    const float* p0 = raw + r0 * RAWX + (RAW_SHIFT + lx) * 3;
                    const float* p1 = p0 + RAWX;
                    const float u[12] = {p0[0], p0[1], p0[2], p0[3], p0[4], p0[5],
                                         p1[3], p1[4], p1[5], p1[0], p1[1], p1[2]};
#pragma unroll
                    for (int i = 0; i < 12; ++i) {
                        hv[i] = to_tf32(u[i]);
                        lv[i] = to_tf32(__fsub_rn(u[i], hv[i]));
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 12; ++i) { hv[i] = 0.f; lv[i] = 0.f; }
                }
                unsigned char* Ab = smem + OFF_A + b * A_STRIDE;
                const int off = (m >> 3) * SBO + (3 * h) * LBO + (m & 7) * 16;
#pragma unroll
                for (int g = 0; g < 3; ++g) {
                    *reinterpret_cast<float4*>(Ab + off + g * LBO) = make_float4(hv[4 * g], hv[4 * g + 1], hv[4 * g + 2], hv[4 * g + 3]);
                    *reinterpret_cast<float4*>(Ab + A_BYTES + off + g * LBO) = make_float4(lv[4 * g], lv[4 * g + 1], lv[4 * g + 2], lv[4 * g + 3]);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(B_AFULL(b));
            }
        }
    } else if (warp == ISSUE_WARP) {
        // ===== MMA issuer: D = A_lo K_hi + A_hi K_lo + A_hi K_hi in one accumulator =====
        if (lane == 0) {
            uint32_t ph_afull = 0u, ph_dempty = (1u << NDB) - 1u;
            const uint32_t bB = smem_u32(smem + OFF_B);
            const int total = ntile_cta * NMT;
            for (int mt = 0; mt < total && ok; ++mt) {
                const int b = mt & 1, db = mt % NDB;
                ok = mbar_wait(B_AFULL(b), PH(ph_afull, b)) && mbar_wait(B_DEMPTY(db), PH(ph_dempty, db));
                FLIP(ph_afull, b);
                FLIP(ph_dempty, db);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a_hi = smem_u32(smem + OFF_A + b * A_STRIDE), a_lo = a_hi + A_BYTES;
                const uint32_t d = tmem + (uint32_t)db * ACC_COLS;
#pragma unroll
                for (int ks = 0; ks < KDIM / 8; ++ks) {       // three K=8 steps (2 core matrices each)
                    const uint32_t koff = ks * 2 * LBO;
                    // the two small correction products first, then the main one
                    mma_tf32(d, make_desc(a_lo + koff), make_desc(bB + koff), kIdescN48, ks > 0);
                    mma_tf32(d, make_desc(a_hi + koff), make_desc(bB + B_LO_OFF + koff), kIdescN48, 1);
                    mma_tf32(d, make_desc(a_hi + koff), make_desc(bB + koff), kIdescN48, 1);
                }
                mma_commit(B_DFULL(db));
                mma_commit(B_AEMPTY(b));
            }
        }
    } else {
        // ===== warps 9-15: TMA, TMEM drain (12-15), ordered gather, update ======
        const int gt = tid - UPD_WARP0 * 32;                  // 0..223
        uint32_t ph_tma = 0u, ph_dfull = 0u, ph_own = 0;
        uint32_t pending = 0u;
        bool pending_own = ntile_cta > 0;
        if (gt == 0) {
            for (int it = 0; it < 2 && it < ntile_cta; ++it) issue_tile(blockIdx.x + it * gridDim.x, it);
            if (ntile_cta > 0) issue_owned(blockIdx.x);
        }
        for (int it = 0; it < 2 && it < ntile_cta; ++it) pending |= 1u << it;
        for (int it = 0, mt = 0; it < ntile_cta && ok; ++it) {
            const int tile = blockIdx.x + it * gridDim.x;
            const int buf = it & 1;
            const TileOrigin o = tile_origin(v, tile);
            const int tl0 = v.tl_ptr[tile], tl1 = v.tl_ptr[tile + 1];     // used at the end of the tile
            const unsigned char* tt = smem + OFF_TT + buf * TT_STRIDE;
            const float* raw = reinterpret_cast<const float*>(tt);
            const float* tlam = reinterpret_cast<const float*>(tt + TT_LAM);
            const float* tmu = reinterpret_cast<const float*>(tt + TT_MU);
            ok = mbar_wait(B_TMA(buf), PH(ph_tma, buf));
            FLIP(ph_tma, buf);
            pending &= ~(1u << buf);
            if (warp >= EPI_WARP0) {
                const int q = warp - EPI_WARP0;                   // TMEM lane quarter
                for (int t = 0; t < NMT; ++t, ++mt) {
                    const int b = mt % NDB;
                    ok = ok && mbar_wait(B_DFULL(b), PH(ph_dfull, b));
                    FLIP(ph_dfull, b);
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t row = tmem + (uint32_t)b * ACC_COLS + ((uint32_t)(q * 32) << 16);
                    const int le = t * 128 + q * 32 + lane;
                    const int lx = le % EX, lr = min(le, NEL - 1) / EX;          // lr = lz*EY + ly
                    const float l = tlam[lr * LMX + LM_SHIFT + lx], mu = tmu[lr * LMX + LM_SHIFT + lx];
                    // cols 0-23 K_lambda u, 24-47 K_mu u
                    float dv[48];
#pragma unroll
                    for (int g = 0; g < 6; ++g) tmem_ld<8>(row + 8 * g, dv + 8 * g);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    mbar_arrive(B_DEMPTY(b));
                    if (le < NEL) {
#pragma unroll
                        for (int jj = 0; jj < 24; ++jj) sF[le * FSTRIDE + jj] = l * dv[jj] + mu * dv[24 + jj];
                    }
                }
            } else {
                mt += NMT;
            }
            // all element forces of this tile are in sF (group barrier; ok made uniform);
            // the owned-node state of this tile has landed
            ok = ok && mbar_wait(b_own, ph_own);
            ph_own ^= 1;
            pending_own = false;
            ok = group_and(ok);
            if (!ok) break;

            // -- ordered gather and compensated update of the owned nodes -----
            const float* tulc = reinterpret_cast<const float*>(smem + OFF_OWN + OWN_ULC);
            const float* tuhp = reinterpret_cast<const float*>(smem + OFF_OWN + OWN_UHP);
            const float* tulp = reinterpret_cast<const float*>(smem + OFF_OWN + OWN_ULP);
            const float* tcd = reinterpret_cast<const float*>(smem + OFF_OWN + OWN_CD);
            for (int nd = gt; nd < TX * TY * TZ; nd += NUPD) {
                const int ox = nd & 7, oy = (nd >> 3) & 7, oz = nd >> 6;
                const int gx = o.x0 + ox, gy = o.y0 + oy, gz = o.z0 + oz;
                if (gx >= nxn || gy >= nyn || gz >= nzn) continue;
                // (element offset, local node) in ascending element-tag order
                const int sel[8][4] = {{0, 0, 0, 6}, {1, 0, 0, 7}, {0, 1, 0, 5}, {1, 1, 0, 4},
                                       {0, 0, 1, 2}, {1, 0, 1, 3}, {0, 1, 1, 1}, {1, 1, 1, 0}};
                float f[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int s2 = 0; s2 < 8; ++s2) {
                    const int le = ((oz + sel[s2][2]) * EY + (oy + sel[s2][1])) * EX + (ox + sel[s2][0]);
                    const float* fe = sF + le * FSTRIDE + sel[s2][3] * 3;
                    f[0] += fe[0]; f[1] += fe[1]; f[2] += fe[2];
                }
                const size_t gbase = ((((size_t)o.inst * nzn + gz) * nyn + gy) * v.pitch) + (size_t)gx * 3;
                const int ob = (oz * TY + oy) * (TX * 3) + ox * 3;
                const float* ah = raw + ((oz + 1) * HY + (oy + 1)) * RAWX + (RAW_SHIFT + ox + 1) * 3;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float inc = -tcd[ob + c] * f[c];
                    float dh, dl2, Dh, Dl, nh, nl;
                    df_add(ah[c], tulc[ob + c], -tuhp[ob + c], -tulp[ob + c], dh, dl2);   // u_n - u_{n-1}
                    df_add(dh, dl2, inc, 0.f, Dh, Dl);                                    // + (dt^2/m)(-f_int)
                    df_add(ah[c], tulc[ob + c], Dh, Dl, nh, nl);                          // u_{n+1}
                    v.uh_prev[gbase + c] = nh;
                    v.ul_prev[gbase + c] = nl;
                }
            }
            asm volatile("bar.sync 2, %0;" :: "r"(NUPD) : "memory");   // element forces and the tile buffers are free
            if (gt == 0 && it + 1 < ntile_cta) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_owned(blockIdx.x + (it + 1) * gridDim.x);
            }
            if (it + 1 < ntile_cta) pending_own = true;
            // -- external loads on this tile's dofs: (dt^2/m) f_ext(k) -------
            if (tl1 > tl0) {
                for (int j2 = tl0 + gt; j2 < tl1; j2 += NUPD) {
                    double fx = 0.0;
                    for (int e = v.ld_ptr[j2]; e < v.ld_ptr[j2 + 1]; ++e) {
                        const int sidx = v.ld_ser[e];
                        const int b0 = v.s_ptr[sidx], n = v.s_ptr[sidx + 1] - b0;
                        fx += v.ld_coef[e] * ((v.k >= 0 && v.k < n) ? v.s_val[b0 + v.k] : 0.0);
                    }
                    const long long d = v.ld_dof[j2];
                    const double inc = (double)v.cdof[d] * fx;
                    const float ih = (float)inc, il = (float)(inc - (double)ih);
                    float nh, nl;
                    df_add(v.uh_prev[d], v.ul_prev[d], ih, il, nh, nl);
                    v.uh_prev[d] = nh;
                    v.ul_prev[d] = nl;
                }
            }
            // this tile's buffer is free: bring in the tile after next
            if (gt == 0 && it + 2 < ntile_cta) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_tile(blockIdx.x + (it + 2) * gridDim.x, buf);
            }
            if (it + 2 < ntile_cta) pending |= 1u << buf;
        }
        if (!ok) {
            if (gt == 0) atomicOr(v.status, 1);
            for (int b = 0; b < 2; ++b)            // never leave with a TMA copy in flight
                if ((pending >> b) & 1u) mbar_wait(B_TMA(b), PH(ph_tma, b));
            if (pending_own) mbar_wait(b_own, ph_own);
        }
    }
    if (!ok) atomicOr(v.status, 1);

    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// V and A of the last step from u_{n+1}, u_n, u_{n-1} (CentralDifference.cpp:141-144),
// evaluated in FP64 from the compensated pairs (once per run).
__global__ void k_cdx_va(const float* nh, const float* nl, const float* ch, const float* cl, const float* ph,
                         const float* pl, double* V, double* A, long long n, double inv_2dt, double inv_dt2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double un = (double)nh[i] + (double)nl[i];
    const double u = (double)ch[i] + (double)cl[i];
    const double up = (double)ph[i] + (double)pl[i];
    const double dU = un - u;
    V[i] = inv_2dt * (u + dU - up);
    A[i] = inv_dt2 * (dU - u + up);
}

// FP64 total-dof displacement of every instance from the padded compensated
// pairs: out[b][t] = hi + lo at the padded position of total dof t = node*3 + c.
__global__ void k_cdx_hist(const float* __restrict__ uh, const float* __restrict__ ul, double* __restrict__ out,
                           long long ntotal, int nxn, int nyn, int pitch, long long per, int ninst) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntotal * ninst) return;
    const long long b = i / ntotal, t = i - b * ntotal;
    const long long n = t / 3;
    const int c = (int)(t - n * 3);
    const long long x = n % nxn, y = (n / nxn) % nyn, z = n / ((long long)nxn * nyn);
    const long long p = b * per + (z * nyn + y) * pitch + x * 3 + c;
    out[i] = (double)uh[p] + (double)ul[p];
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
    int pitch = 0;                       // floats per padded x-row (multiple of 4)
    long long nstate = 0;                // padded state length (all instances)
    int ntx = 0, nty = 0, ntz = 0, ntiles = 0, grid = 0;
    double dt = 0;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    float* uh[2] = {nullptr, nullptr};   // compensated displacement pairs (hi, lo), padded rows
    float* ul[2] = {nullptr, nullptr};
    float* ph_copy = nullptr;            // u_{n-1} kept for V/A of the last step
    float* pl_copy = nullptr;
    double* V = nullptr;
    double* A = nullptr;
    float *lam = nullptr, *mu = nullptr, *cdof = nullptr, *bop = nullptr;
    int* status = nullptr;
    int *tl_ptr = nullptr, *ld_ptr = nullptr, *ld_ser = nullptr, *s_ptr = nullptr;
    long long* ld_dof = nullptr;
    double *ld_coef = nullptr, *s_val = nullptr;
    int pe = 0;                          // floats per padded element row of lambda/mu
    CUtensorMap tmap[2];                 // halo maps of uh[0], uh[1]
    CUtensorMap own_uh[2], own_ul[2];    // owned-node maps of uh[*], ul[*]
    CUtensorMap own_cd;                  // owned-node map of dt^2/m
    CUtensorMap tmap_lam, tmap_mu;
    std::vector<long long> pad_index;    // total dof (node*3+c) -> padded position, one instance
    int cur = 0;                         // index of u_n in uh/ul
    int64_t launches = 0, launches_last = 0;
    bool va_valid = false;
    // history: two device chunks, filled on `stream`, drained on `copy_stream`
    double* hist[2] = {nullptr, nullptr};
    int hist_cap = 0;                    // steps per chunk
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t filled[2] = {nullptr, nullptr}, drained[2] = {nullptr, nullptr};

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
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        for (void* p : allocs) cudaFree(p);
        for (int i = 0; i < 2; ++i) {
            if (hist[i]) cudaFree(hist[i]);
            if (filled[i]) cudaEventDestroy(filled[i]);
            if (drained[i]) cudaEventDestroy(drained[i]);
        }
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (stream) cudaStreamDestroy(stream);
    }
};

// 4D tiled map {pitch, ny, nz, ninst} floats with box {bx, by, bz, 1};
// out-of-range elements read as zero.
static int make_map(float* base, int pitch, int ny, int nz, int ninst, int bx, int by, int bz, CUtensorMap* map) {
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
    const cuuint64_t dims[4] = {(cuuint64_t)pitch, (cuuint64_t)ny, (cuuint64_t)nz, (cuuint64_t)ninst};
    const cuuint64_t strides[3] = {(cuuint64_t)pitch * 4, (cuuint64_t)pitch * 4 * ny, (cuuint64_t)pitch * 4 * ny * nz};
    const cuuint32_t box[4] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz, 1};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return SVL_ERR_CUDA; }
    return SVL_OK;
}

static int cdx_check_instance(const svl_grid_spec* g, const HostModel& m, int inst) {
    const int nx = g->ne[0], ny = g->ne[1], nz = g->ne[2];
    const long long nn = (long long)(nx + 1) * (ny + 1) * (nz + 1);
    if (m.etype != SVL_ELEM_LIN3DHEXA8 || m.ndim != 3) { set_error("instance %d: the structured path needs lin3DHexa8", inst); return SVL_ERR_UNSUPPORTED; }
    if (m.nnode != nn || m.nelem != (long long)nx * ny * nz) { set_error("instance %d does not match the grid size", inst); return SVL_ERR_INVALID; }
    if (m.nconstraint) { set_error("instance %d: constraints are not supported on the structured path", inst); return SVL_ERR_UNSUPPORTED; }
    if (!m.lumped) { set_error("instance %d: the explicit path needs a lumped mass", inst); return SVL_ERR_UNSUPPORTED; }
    if (m.has_pml()) { set_error("instance %d: PML elements are served by svl_xnm_create", inst); return SVL_ERR_UNSUPPORTED; }
    if (!m.ray.empty()) { set_error("instance %d: Rayleigh damping is served by the general path (svl_cd_create)", inst); return SVL_ERR_UNSUPPORTED; }
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

static void split_pair(double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// Device pair (hi, lo) of instance `inst` -> FP64 total-dof vector.
static int fetch_pair(svl_cdx* h, const float* dh, const float* dl, int inst, double* out) {
    const size_t per = h->nstate / h->ninst;
    std::vector<float> hi(per), lo(per);
    CUDA_TRY(cudaMemcpyAsync(hi.data(), dh + (size_t)inst * per, per * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaMemcpyAsync(lo.data(), dl + (size_t)inst * per, per * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (long long t = 0; t < h->ntotal; ++t) {
        const long long p = h->pad_index[t];
        out[t] = (double)hi[p] + (double)lo[p];
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
    const int nxn = h->nx + 1, nyn = h->ny + 1, nzn = h->nz + 1;
    h->nn = (long long)nxn * nyn * nzn;
    h->ne = (long long)h->nx * h->ny * h->nz;
    h->ntotal = h->nn * 3;
    h->pitch = (nxn * 3 + 3) / 4 * 4;
    const long long per = (long long)h->pitch * nyn * nzn;
    h->nstate = per * ninst;
    h->ntx = (nxn + TX - 1) / TX; h->nty = (nyn + TY - 1) / TY; h->ntz = (nzn + TZ - 1) / TZ;
    const long long ntiles = (long long)h->ntx * h->nty * h->ntz * ninst;
    if (ntiles > INT32_MAX || h->nstate > ((long long)1 << 40)) { set_error("grid too large"); return fail(SVL_ERR_INVALID); }
    h->ntiles = (int)ntiles;
    h->dt = opts->dt;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) { set_error("cudaStreamCreate failed"); return fail(SVL_ERR_CUDA); }
    h->pad_index.resize(h->ntotal);
    for (long long n = 0; n < h->nn; ++n) {
        const long long x = n % nxn, y = (n / nxn) % nyn, z = n / ((long long)nxn * nyn);
        for (int c = 0; c < 3; ++c) h->pad_index[n * 3 + c] = (z * nyn + y) * h->pitch + x * 3 + c;
    }

    h->pe = (h->nx + 8 + 3) / 4 * 4;                  // row padding keeps TMA strides 16-byte multiples
    const size_t lm_per = (size_t)h->pe * h->ny * h->nz;
    std::vector<float> lam(lm_per * ninst, 0.f), mu(lm_per * ninst, 0.f), cdof((size_t)h->nstate, 0.f);
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
        if (b == 0) {
            // reference matrices of the (uniform) element: K = lambda K_lambda + mu K_mu
            for (int q = 0; q < 8; ++q) {
                double dNx[8][3], N[8];
                const double w = gp_factor(m, 0, gp_geometry(m, 0, q, dNx, N));
                double div[24], B[6][24];
                for (int i2 = 0; i2 < 24; ++i2) { div[i2] = 0; for (int r = 0; r < 6; ++r) B[r][i2] = 0; }
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
                for (int r1 = 0; r1 < 24; ++r1)
                    for (int c1 = 0; c1 < 24; ++c1) {
                        Klam[r1 * 24 + c1] += w * div[r1] * div[c1];
                        double acc = 0;
                        for (int r = 0; r < 6; ++r) acc += B[r][r1] * D[r] * B[r][c1];
                        Kmu[r1 * 24 + c1] += w * acc;
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
            const double* pr = m.param(e);
            const double E = pr[0], nu = pr[1];
            const int ex = e % h->nx, ey = (e / h->nx) % h->ny, ez = e / (h->nx * h->ny);
            const size_t li = (size_t)b * lm_per + ((size_t)ez * h->ny + ey) * h->pe + ex;
            lam[li] = (float)(E * nu / (1.0 - 2.0 * nu) / (1.0 + nu));
            mu[li] = (float)(E / (2.0 * (1.0 + nu)));
        }
        std::vector<double> M;
        lumped_mass_diag(m, opts->mtol, M);
        for (long long t = 0; t < h->ntotal; ++t) {
            const bool fixed = m.fdof[t] < 0;
            if (!fixed && !(M[t] > 0)) { set_error("instance %d: free dof %lld has no mass", b, t); return fail(SVL_ERR_INVALID); }
            cdof[(size_t)b * per + h->pad_index[t]] = fixed ? 0.0f : (float)(dt2 / M[t]);
        }
        if (loads) {
            const svl_load_desc& L = loads[b];
            if (L.ndrm > 0) { set_error("instance %d: domain-reduction loads are served by svl_cd_create", b); return fail(SVL_ERR_UNSUPPORTED); }
            if (L.nsupport > 0) { set_error("instance %d: support motion is not supported on the structured path", b); return fail(SVL_ERR_UNSUPPORTED); }
            const int soff = (int)s_ptr.size() - 1;
            for (int sidx = 0; sidx < L.nseries; ++sidx) {
                const int n = L.series_ptr[sidx + 1] - L.series_ptr[sidx];
                if (n < 0) { set_error("bad series_ptr"); return fail(SVL_ERR_INVALID); }
                s_val.insert(s_val.end(), L.series_val + L.series_ptr[sidx], L.series_val + L.series_ptr[sidx + 1]);
                s_ptr.push_back((int)s_val.size());
            }
            for (int i2 = 0; i2 < L.nforce; ++i2) {
                if (L.force_dof[i2] < 0 || L.force_dof[i2] >= h->ntotal || L.force_series[i2] < 0 || L.force_series[i2] >= L.nseries) {
                    set_error("instance %d: load entry %d out of range", b, i2); return fail(SVL_ERR_INVALID);
                }
                fdof.push_back((long long)b * h->ntotal + L.force_dof[i2]);
                fser.push_back(soff + L.force_series[i2]);
                fcoef.push_back(L.force_coef[i2]);
            }
        }
    }
    // B operand image, canonical K-major layout, 96 rows:
    // [K_lambda hi; K_mu hi; K_lambda lo; K_mu lo] (24 rows each)
    std::vector<float> bop(B_BYTES / 4, 0.f);
    for (int n = 0; n < 48; ++n)
        for (int k = 0; k < 24; ++k) {
            const double val = n < 24 ? Klam[n * 24 + k] : Kmu[(n - 24) * 24 + k];
            const float hi = host_tf32(val);
            const float lo = host_tf32(val - (double)hi);
            const int nl = n + 48;
            bop[(n >> 3) * (SBO / 4) + (k >> 2) * (LBO / 4) + (n & 7) * 4 + (k & 3)] = hi;
            bop[(nl >> 3) * (SBO / 4) + (k >> 2) * (LBO / 4) + (nl & 7) * 4 + (k & 3)] = lo;
        }
    // loads: unique dofs (entries kept in input order), grouped by the tile owning the node
    std::vector<int> order(fdof.size());
    for (size_t i2 = 0; i2 < order.size(); ++i2) order[i2] = (int)i2;
    auto tile_of = [&](long long gdof) {
        const long long b = gdof / h->ntotal, t = gdof % h->ntotal, n = t / 3;
        const long long x = n % nxn, y = (n / nxn) % nyn, z = n / ((long long)nxn * nyn);
        return (((b * h->ntz + z / TZ) * h->nty + y / TY) * h->ntx + x / TX);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const long long ta = tile_of(fdof[a]), tc = tile_of(fdof[c]);
        return ta < tc || (ta == tc && fdof[a] < fdof[c]);
    });
    std::vector<int> tl_ptr(h->ntiles + 1, 0), ld_ptr(1, 0), ld_ser;
    std::vector<long long> ld_dof;
    std::vector<double> ld_coef;
    long long last = -1;
    for (int j2 : order) {
        if (fdof[j2] != last) {
            if (last >= 0) ld_ptr.push_back((int)ld_ser.size());
            const long long b = fdof[j2] / h->ntotal, t = fdof[j2] % h->ntotal;
            ld_dof.push_back(b * per + h->pad_index[t]);
            tl_ptr[tile_of(fdof[j2]) + 1]++;
            last = fdof[j2];
        }
        ld_ser.push_back(fser[j2]);
        ld_coef.push_back(fcoef[j2]);
    }
    if (last >= 0) ld_ptr.push_back((int)ld_ser.size());
    for (int t = 0; t < h->ntiles; ++t) tl_ptr[t + 1] += tl_ptr[t];

    int st;
    const size_t ns = (size_t)h->nstate;
    if ((st = h->alloc(ns, &h->uh[0])) || (st = h->alloc(ns, &h->uh[1])) || (st = h->alloc(ns, &h->ul[0])) ||
        (st = h->alloc(ns, &h->ul[1])) || (st = h->alloc(ns, &h->ph_copy)) || (st = h->alloc(ns, &h->pl_copy)) ||
        (st = h->alloc(ns, &h->V)) || (st = h->alloc(ns, &h->A)) || (st = h->upload(lam, &h->lam)) ||
        (st = h->upload(mu, &h->mu)) || (st = h->upload(cdof, &h->cdof)) || (st = h->upload(bop, &h->bop)) ||
        (st = h->alloc(1, &h->status)) || (st = h->upload(tl_ptr, &h->tl_ptr)) || (st = h->upload(ld_dof, &h->ld_dof)) ||
        (st = h->upload(ld_ptr, &h->ld_ptr)) || (st = h->upload(ld_ser, &h->ld_ser)) || (st = h->upload(ld_coef, &h->ld_coef)) ||
        (st = h->upload(s_ptr, &h->s_ptr)) || (st = h->upload(s_val, &h->s_val)))
        return fail(st);
    if ((st = make_map(h->uh[0], h->pitch, nyn, nzn, ninst, RAWX, HY, HZ, &h->tmap[0])) ||
        (st = make_map(h->uh[1], h->pitch, nyn, nzn, ninst, RAWX, HY, HZ, &h->tmap[1])) ||
        (st = make_map(h->lam, h->pe, h->ny, h->nz, ninst, LMX, EY, EZ, &h->tmap_lam)) ||
        (st = make_map(h->mu, h->pe, h->ny, h->nz, ninst, LMX, EY, EZ, &h->tmap_mu)) ||
        (st = make_map(h->uh[0], h->pitch, nyn, nzn, ninst, TX * 3, TY, TZ, &h->own_uh[0])) ||
        (st = make_map(h->uh[1], h->pitch, nyn, nzn, ninst, TX * 3, TY, TZ, &h->own_uh[1])) ||
        (st = make_map(h->ul[0], h->pitch, nyn, nzn, ninst, TX * 3, TY, TZ, &h->own_ul[0])) ||
        (st = make_map(h->ul[1], h->pitch, nyn, nzn, ninst, TX * 3, TY, TZ, &h->own_ul[1])) ||
        (st = make_map(h->cdof, h->pitch, nyn, nzn, ninst, TX * 3, TY, TZ, &h->own_cd)))
        return fail(st);
    if (cudaFuncSetAttribute(k_cdx_step, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess) {
        set_error("cannot set %d bytes of dynamic shared memory", SMEM_BYTES); return fail(SVL_ERR_CUDA);
    }
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    h->grid = std::min(h->ntiles, sms);      // persistent: one CTA per SM
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) { set_error("upload failed"); return fail(SVL_ERR_CUDA); }
    *out = h;
    return SVL_OK;
}

int svl_cdx_set_initial(svl_cdx* h, int32_t inst, const double* U0, const double* V0, const double* A0) {
    if (!h || inst < 0 || inst >= h->ninst) { set_error("bad handle or instance"); return SVL_ERR_INVALID; }
    const size_t per = (size_t)(h->nstate / h->ninst);
    std::vector<float> hi(per, 0.f), lo(per, 0.f), phi(per, 0.f), plo(per, 0.f);
    for (long long t = 0; t < h->ntotal; ++t) {
        const double u = U0 ? U0[t] : 0.0, vv = V0 ? V0[t] : 0.0, a = A0 ? A0[t] : 0.0;
        const double up = u - h->dt * vv + h->dt * h->dt / 2.0 * a;
        const long long p = h->pad_index[t];
        split_pair(u, hi[p], lo[p]);
        split_pair(up, phi[p], plo[p]);
    }
    const size_t off = (size_t)inst * per;
    CUDA_TRY(cudaMemcpyAsync(h->uh[h->cur] + off, hi.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->ul[h->cur] + off, lo.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->uh[1 - h->cur] + off, phi.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->ul[1 - h->cur] + off, plo.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->va_valid = false;
    return SVL_OK;
}

static int cdx_step(svl_cdx* h, int k, bool want_va) {
    CdxView v;
    v.nx = h->nx; v.ny = h->ny; v.nz = h->nz; v.ninst = h->ninst;
    v.pitch = h->pitch; v.ntx = h->ntx; v.nty = h->nty; v.ntz = h->ntz; v.ntiles = h->ntiles;
    v.uh_prev = h->uh[1 - h->cur]; v.ul_prev = h->ul[1 - h->cur];
    v.cdof = h->cdof; v.bop = h->bop;
    v.tl_ptr = h->tl_ptr; v.ld_dof = h->ld_dof; v.ld_ptr = h->ld_ptr; v.ld_ser = h->ld_ser; v.ld_coef = h->ld_coef;
    v.s_ptr = h->s_ptr; v.s_val = h->s_val;
    v.k = k;
    v.status = h->status;
    const size_t ns = (size_t)h->nstate;
    if (want_va) {
        CUDA_TRY(cudaMemcpyAsync(h->ph_copy, v.uh_prev, ns * 4, cudaMemcpyDeviceToDevice, h->stream));
        CUDA_TRY(cudaMemcpyAsync(h->pl_copy, v.ul_prev, ns * 4, cudaMemcpyDeviceToDevice, h->stream));
    }
    k_cdx_step<<<h->grid, NTHREADS, SMEM_BYTES, h->stream>>>(h->tmap[h->cur], h->tmap_lam, h->tmap_mu, h->own_ul[h->cur],
                                                             h->own_uh[1 - h->cur], h->own_ul[1 - h->cur], h->own_cd, v);
    ++h->launches;
    if (want_va) {
        k_cdx_va<<<(unsigned)((ns + 255) / 256), 256, 0, h->stream>>>(v.uh_prev, v.ul_prev, h->uh[h->cur], h->ul[h->cur], h->ph_copy,
                                                                   h->pl_copy, h->V, h->A, (long long)ns,
                                                                   1.0 / 2.0 / h->dt, 1.0 / h->dt / h->dt);
        ++h->launches;
    }
    CUDA_TRY(cudaGetLastError());
    h->cur = 1 - h->cur;
    return SVL_OK;
}

static int cdx_status(svl_cdx* h) {
    int status = 0;
    CUDA_TRY(cudaMemcpyAsync(&status, h->status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (status) { set_error("tensor-core step gave up waiting on a barrier (status %d)", status); return SVL_ERR_CUDA; }
    return SVL_OK;
}

// Enqueues steps [s0, s0 + n) of a run on the compute stream, writing each
// step's FP64 fields into history chunk `slot`.
static int cdx_fill_chunk(svl_cdx* h, int k_first, int s0, int n, int nsteps, int slot) {
    const long long per_step = h->ntotal * h->ninst;
    CUDA_TRY(cudaStreamWaitEvent(h->stream, h->drained[slot], 0));       // the chunk's previous copy is done
    for (int i = 0; i < n; ++i) {
        const int s = s0 + i;
        TRY(cdx_step(h, k_first + s, s == nsteps - 1));
        k_cdx_hist<<<(unsigned)((per_step + 255) / 256), 256, 0, h->stream>>>(
            h->uh[h->cur], h->ul[h->cur], h->hist[slot] + (size_t)i * per_step, h->ntotal, h->nx + 1, h->ny + 1, h->pitch,
            h->nstate / h->ninst, h->ninst);
        ++h->launches;
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(h->filled[slot], h->stream));
    return SVL_OK;
}

int svl_cdx_run(svl_cdx* h, int32_t k_first, int32_t nsteps, double* U_hist) {
    if (!h || nsteps < 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    const int64_t l0 = h->launches;
    if (!U_hist) {
        for (int s = 0; s < nsteps; ++s) TRY(cdx_step(h, k_first + s, s == nsteps - 1));
    } else if (nsteps > 0) {
        // device-side FP64 conversion into two chunk buffers; the copy of chunk
        // c (on copy_stream) overlaps the computation of chunk c + 1
        const long long per_step = h->ntotal * h->ninst;
        const int chunk = (int)std::max<long long>(1, std::min<long long>(nsteps, (256ll << 20) / (per_step * 8)));
        if (h->hist_cap < chunk) {
            CUDA_TRY(cudaStreamSynchronize(h->stream));
            if (h->copy_stream) CUDA_TRY(cudaStreamSynchronize(h->copy_stream));
            for (int i = 0; i < 2; ++i) {
                if (h->hist[i]) cudaFree(h->hist[i]);
                h->hist[i] = nullptr;
            }
            h->hist_cap = 0;
            for (int i = 0; i < 2; ++i)
                if (cudaMalloc(&h->hist[i], (size_t)chunk * per_step * sizeof(double)) != cudaSuccess) {
                    set_error("history buffer allocation failed");
                    return SVL_ERR_NOMEM;
                }
            if (!h->copy_stream) {
                CUDA_TRY(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
                for (int i = 0; i < 2; ++i) {
                    CUDA_TRY(cudaEventCreateWithFlags(&h->filled[i], cudaEventDisableTiming));
                    CUDA_TRY(cudaEventCreateWithFlags(&h->drained[i], cudaEventDisableTiming));
                    CUDA_TRY(cudaEventRecord(h->drained[i], h->copy_stream));
                }
            }
            h->hist_cap = chunk;
        }
        const int nch = (nsteps + chunk - 1) / chunk;
        TRY(cdx_fill_chunk(h, k_first, 0, std::min(chunk, nsteps), nsteps, 0));
        for (int c = 0; c < nch; ++c) {
            const int s0 = c * chunk, n = std::min(chunk, nsteps - s0), slot = c & 1;
            if (c + 1 < nch) {
                const int s1 = s0 + chunk;
                TRY(cdx_fill_chunk(h, k_first, s1, std::min(chunk, nsteps - s1), nsteps, slot ^ 1));
            }
            CUDA_TRY(cudaStreamWaitEvent(h->copy_stream, h->filled[slot], 0));
            CUDA_TRY(cudaMemcpyAsync(U_hist + (size_t)s0 * per_step, h->hist[slot], (size_t)n * per_step * sizeof(double),
                                     cudaMemcpyDeviceToHost, h->copy_stream));
            CUDA_TRY(cudaEventRecord(h->drained[slot], h->copy_stream));
        }
        CUDA_TRY(cudaStreamSynchronize(h->copy_stream));
    }
    h->va_valid = nsteps > 0;
    h->launches_last = h->launches - l0;
    return cdx_status(h);
}

int svl_cdx_run_timed(svl_cdx* h, int32_t k_first, int32_t nsteps, float* ms) {
    if (!h || !ms) { set_error("bad argument"); return SVL_ERR_INVALID; }
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    const int64_t l0 = h->launches;
    CUDA_TRY(cudaEventRecord(a, h->stream));
    for (int s = 0; s < nsteps; ++s) TRY(cdx_step(h, k_first + s, false));
    CUDA_TRY(cudaEventRecord(b, h->stream));
    CUDA_TRY(cudaEventSynchronize(b));
    CUDA_TRY(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    h->launches_last = h->launches - l0;
    h->va_valid = false;
    return cdx_status(h);
}

int svl_cdx_get(svl_cdx* h, int32_t inst, int32_t which, double* out) {
    if (!h || !out || inst < 0 || inst >= h->ninst) { set_error("bad argument"); return SVL_ERR_INVALID; }
    if (which < 0 || which > 2) { set_error("which must be 0, 1 or 2"); return SVL_ERR_INVALID; }
    if (which == 0) return fetch_pair(h, h->uh[h->cur], h->ul[h->cur], inst, out);
    if (!h->va_valid) { set_error("V/A are only available after svl_cdx_run"); return SVL_ERR_INVALID; }
    const size_t per = (size_t)(h->nstate / h->ninst);
    std::vector<double> tmp(per);
    CUDA_TRY(cudaMemcpyAsync(tmp.data(), (which == 1 ? h->V : h->A) + (size_t)inst * per, per * 8, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    for (long long t = 0; t < h->ntotal; ++t) out[t] = tmp[h->pad_index[t]];
    return SVL_OK;
}

int svl_cdx_set_ctas(svl_cdx* h, int32_t ctas) {
    if (!h || ctas < 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int cap = ctas == 0 ? sms : std::min(ctas, sms);
    h->grid = std::max(1, std::min(h->ntiles, cap));
    return SVL_OK;
}

int svl_cdx_get_ctas(svl_cdx* h, int32_t* ctas) {
    if (!h || !ctas) { set_error("bad argument"); return SVL_ERR_INVALID; }
    *ctas = h->grid;
    return SVL_OK;
}

int svl_cdx_launch_count(svl_cdx* h, int64_t* launches) {
    if (!h || !launches) { set_error("bad argument"); return SVL_ERR_INVALID; }
    *launches = h->launches_last;
    return SVL_OK;
}

void svl_cdx_destroy(svl_cdx* h) { delete h; }

}  // extern "C"
