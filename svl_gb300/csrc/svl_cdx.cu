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
#include <thread>
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
    const int32_t* __restrict__ tiles;   // the schedule: position -> tile of the full enumeration (null: identity)
    float* uh_prev;                      // u_{n-1} (read through TMA), u_{n+1} written here
    float* ul_prev;
    const float* __restrict__ cdof;      // [inst][z][y][pitch]  dt^2/m, 0 on restrained dofs,
                                         // -1 on the displacement dofs of PML nodes
    float* fsol;                         // PML nodes: the solid elements' force sum (same layout), or null
    const float* __restrict__ bop;       // [B_ROWS x 24] hi then lo operand image
    float kscale;                        // the B image holds K / kscale (1: hi/lo split of K)
    int b_exact;                         // 1: the B image is exact in TF32 (its lo half zero)
    // external loads grouped by tile, then by dof
    const int* __restrict__ tl_ptr;      // [full tiles + 1] into the unique-dof arrays
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
    int r = v.tiles ? v.tiles[tile] : tile;
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
        // half an element row of M-tile t from the halo: TF32 hi and lo parts
        auto build_row = [&](const float* raw, int t, float (&hv)[12], float (&lv)[12]) {
            const int le = t * 128 + m;
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
        };
        for (int it = 0, mt = 0; it < ntile_cta && ok; ++it) {
            const int buf = it & 1;
            ok = mbar_wait(B_TMA(buf), PH(ph_tma, buf));
            FLIP(ph_tma, buf);
            const float* raw = reinterpret_cast<const float*>(smem + OFF_TT + buf * TT_STRIDE);
            // the row of the next M-tile is read and converted while the
            // current one's MMA runs (the halo buffer stays until this tile's
            // update, which needs every M-tile's product first)
            float hv[12], lv[12];
            build_row(raw, 0, hv, lv);
            for (int t = 0; t < NMT && ok; ++t, ++mt) {
                const int b = mt & 1;
                ok = mbar_wait(B_AEMPTY(b), PH(ph_aempty, b));
                FLIP(ph_aempty, b);
                if (!ok) break;
                unsigned char* Ab = smem + OFF_A + b * A_STRIDE;
                const int off = (m >> 3) * SBO + (3 * h) * LBO + (m & 7) * 16;
#pragma unroll
                for (int g = 0; g < 3; ++g) {
                    *reinterpret_cast<float4*>(Ab + off + g * LBO) = make_float4(hv[4 * g], hv[4 * g + 1], hv[4 * g + 2], hv[4 * g + 3]);
                    *reinterpret_cast<float4*>(Ab + A_BYTES + off + g * LBO) = make_float4(lv[4 * g], lv[4 * g + 1], lv[4 * g + 2], lv[4 * g + 3]);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(B_AFULL(b));
                if (t + 1 < NMT) build_row(raw, t + 1, hv, lv);
            }
        }
    } else if (warp == ISSUE_WARP) {
        // ===== MMA issuer: D = A_lo K_hi (+ A_hi K_lo when K is split) + A_hi K_hi in one accumulator =====
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
                    // the small correction products first, then the main one;
                    // an exact B image has no lo half
                    mma_tf32(d, make_desc(a_lo + koff), make_desc(bB + koff), kIdescN48, ks > 0);
                    if (!v.b_exact) mma_tf32(d, make_desc(a_hi + koff), make_desc(bB + B_LO_OFF + koff), kIdescN48, 1);
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
            const int full = v.tiles ? v.tiles[tile] : tile;              // loads are keyed by the full tile id
            const int tl0 = v.tl_ptr[full], tl1 = v.tl_ptr[full + 1];     // used at the end of the tile
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
                    const float l = tlam[lr * LMX + LM_SHIFT + lx] * v.kscale, mu = tmu[lr * LMX + LM_SHIFT + lx] * v.kscale;
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
                    if (tcd[ob + c] < 0.f) {          // PML node: its update is the PML kernels'
                        v.fsol[gbase + c] = f[c];
                        continue;
                    }
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
// FP64 total-dof vector of every instance from the compensated pairs:
// One step's history row: hmap[i] >= 0 is the state position (instance
// offset included) of entry i (instances one after the other, each in its
// own total-dof numbering), -(1 + k) the stress entry k of the PML band's
// arrays (S of the half step after U's time).
__global__ void k_cdx_hist(const float* __restrict__ uh, const float* __restrict__ ul, const float* __restrict__ sh,
                           const float* __restrict__ sl, const long long* __restrict__ hmap, double* __restrict__ out,
                           long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long m = hmap[i];
    if (m >= 0) out[i] = (double)uh[m] + (double)ul[m];
    else out[i] = (double)sh[-m - 1] + (double)sl[-m - 1];
}

// ---- PML band of the mixed path --------------------------------------------
// The explicit staggered PML scheme (displacements at the integer steps, the
// PML stress dofs S at the half steps; lumped N N blocks per node, the
// displacement-stress couplings of PML3DHexa8's C, K, G, PML3DHexa8.cpp:
// 430-712, as element actions) in FP32 arithmetic with the state as
// compensated FP32 pairs.  Each step: k_cdx_step leaves the solid elements'
// force at PML nodes in fsol; k_cdp_fu forms the coupling forces of the PML
// elements on the displacement rows, k_cdp_uu updates u and ubar at the PML
// nodes, k_cdp_fs forms the coupling forces on the stress rows from the new
// u, k_cdp_su updates S and Sbar.  Elements are uniform cubes of side h:
// at Gauss point q, N_a and dN_a/dx are fixed tables and w |J| = (h/2)^3.
struct CdpView {
    int ninst, np, npe;                 // PML nodes and PML elements per instance
    float h, dt;
    long long per;                      // padded state floats per instance
    const int32_t* __restrict__ enode;  // [npe][8] PML node index of each element node
    const float* __restrict__ estr;     // [npe][12] per axis d: a(-g), a(+g), r(-g), r(+g); b = b0 r
    const float* __restrict__ eb0;      // [ninst][npe] b0 of the element's P-wave speed
    const int32_t* __restrict__ ninv;   // [np][8] element slots e*8 + local node in element order, -1 unused
    const long long* __restrict__ npad; // [np] padded offset of the node's displacement in instance 0
    const float* __restrict__ uc;       // [ninst][np][6] 1/d for x y z (0 when restrained), c, Ku, Gu
    const float* __restrict__ scs;      // [ninst][np][12] Dinv, A, KG, Gs as (diagonal, off-diagonal, shear)
    const float* __restrict__ uh;       // u_n pair (padded)
    const float* __restrict__ ul;
    float* uph;                         // u_{n-1} pair in, u_{n+1} out
    float* upl;
    const float* __restrict__ fsol;
    float* ubh; float* ubl;             // [ninst][np][3] ubar pair
    const float* __restrict__ sh;       // S^{n+1/2} pair [ninst][np][6]
    const float* __restrict__ sl;
    float* sph; float* spl;             // S^{n-1/2} in, S^{n+3/2} out
    float* sbh; float* sbl;             // Sbar pair [ninst][np][6]
    float* vsu;                         // [ninst][18][np] displacement rows' inputs: sdot, smid, Sbar (written by k_cdp_su for the next step)
    float* vin;                         // [ninst][9][np] stress rows' inputs: udot, umid, ubar at the half step
    float* feu;                         // [ninst][8][3][npe] element slots (local node, component, element)
    float* fes;                         // [ninst][8][6][npe]
};

// Node rows and element slots are stored component-major ([..][component][node]
// and [..][local node][component][element]): consecutive threads handle
// consecutive nodes / elements, so every load and store of a warp is one
// contiguous run.
constexpr int VSU_K = 18;               // sdot, smid, Sbar x (xx yy zz xy yz xz)
constexpr int VIN_K = 9;                // udot, umid, ubar at the half step x (x y z)
constexpr int SCS_ROW = 12;             // Dinv, A, KG, Gs stress blocks, (diagonal, off-diagonal, shear) each

// Linear shape functions of one axis at its two Gauss points:
// B[q][i] = (1 + s_i xi_q) / 2 with s = (-1, +1), xi = (-g, +g)
// (GaussQuadrature.cpp:303-316 abscissa); B is symmetric.  Their derivative
// is s_i / h at both points, so a derivative along an axis is a difference
// of the two nodes along it.
constexpr float CDP_G = 0.577350269189626f;
constexpr float CDP_P = 0.5f * (1.0f + CDP_G), CDP_Q = 0.5f * (1.0f - CDP_G);

// Element node (the element's own order: (-,-,-) (+,-,-) (+,+,-) (-,+,-),
// then the same at +z) of lexicographic corner l = ir + 2 is + 4 it.
__device__ __forceinline__ constexpr int cdp_lex_node(int l) {
    return (l & 4) | ((l & 2) ? ((l & 1) ? 2 : 3) : (l & 1));
}

// Lexicographic corner with bit `bit` along axis d and index m = i + 2 j
// over the two other axes (in axis order).
__device__ __forceinline__ constexpr int cdp_lex(int d, int m, int bit) {
    return d == 0 ? bit + 2 * m : (d == 1 ? (m & 1) + 2 * bit + 4 * (m >> 1) : m + 4 * bit);
}

// B (x) B over two axes on z[i + 2 j]: the values at the four Gauss points
// (same order) of the bilinear interpolant; B symmetric, so the same map is
// its transpose (Gauss-point values -> nodal sums).
__device__ __forceinline__ void cdp_interp2(float z[4]) {
    const float a0 = CDP_P * z[0] + CDP_Q * z[1], a1 = CDP_Q * z[0] + CDP_P * z[1];
    const float a2 = CDP_P * z[2] + CDP_Q * z[3], a3 = CDP_Q * z[2] + CDP_P * z[3];
    z[0] = CDP_P * a0 + CDP_Q * a2;
    z[2] = CDP_Q * a0 + CDP_P * a2;
    z[1] = CDP_P * a1 + CDP_Q * a3;
    z[3] = CDP_Q * a1 + CDP_P * a3;
}

// Stretching of one element at the two abscissae of each axis.
struct CdpStretch {
    float a[3][2], b[3][2];
};
__device__ __forceinline__ CdpStretch cdp_stretch(const float4 t[3], float b0) {
    CdpStretch s;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        s.a[d][0] = t[d].x; s.a[d][1] = t[d].y; s.b[d][0] = b0 * t[d].z; s.b[d][1] = b0 * t[d].w;
    }
    return s;
}

// Coupling weight of derivative direction d at Gauss point m over the two
// other axes (it does not depend on the abscissa along d), for the C (type
// 0), K (1) and G (2) parts (PML3DHexa8.cpp:952-996; for x: ay az,
// ay bz + az by, by bz).
__device__ __forceinline__ float cdp_w(const CdpStretch& s, int d, int m, int type) {
    const int d1 = d == 0 ? 1 : 0, d2 = d == 2 ? 1 : 2;
    const float a1 = s.a[d1][m & 1], a2 = s.a[d2][m >> 1], b1 = s.b[d1][m & 1], b2 = s.b[d2][m >> 1];
    return type == 0 ? a1 * a2 : (type == 1 ? a1 * b2 + a2 * b1 : b1 * b2);
}

// Stress component (xx yy zz xy yz xz = 0..5) that acts on force component
// j through derivative direction d.
__device__ __forceinline__ constexpr int cdp_fcomp(int d, int j) {
    return d == 0 ? (j == 0 ? 0 : (j == 1 ? 3 : 5)) : (d == 1 ? (j == 0 ? 3 : (j == 1 ? 1 : 4)) : (j == 0 ? 5 : (j == 1 ? 4 : 2)));
}

// Strain component that derivative direction d of displacement component c
// feeds (symmetric pairs share one).
__device__ __forceinline__ constexpr int cdp_scomp(int d, int c) {
    return d == c ? d : (d + c == 1 ? 3 : (d + c == 3 ? 4 : 5));
}

// Coupling forces of the PML elements on the displacement rows,
// C_uS sdot + K_uS smid + G_uS Sbar, one thread per element:
//   f_j = w|J| sum_q sum_d dN_j,d(q) T_d(q),  T_d = C_d sdot + K_d smid + G_d Sbar
// interpolated at Gauss point q.  The shape functions are tensor products and
// dN_j,d is constant along d while the weights of direction d do not depend
// on the abscissa along d, so the sum over the two points along d acts on the
// node values first (their sum), and everything else is a 2 x 2 x 2 map
// over the two other axes (sum factorisation): no per-point 8 x 8 products.
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_cdp_fu(CdpView v) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)v.npe) return;
    const int e = (int)gid;
    int node[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) node[l] = v.enode[(size_t)e * 8 + cdp_lex_node(l)];
    float4 t[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) t[d] = reinterpret_cast<const float4*>(v.estr + (size_t)e * 12)[d];
#pragma unroll 1
    for (int inst = 0; inst < v.ninst; ++inst) {
    const CdpStretch s = cdp_stretch(t, v.eb0[(size_t)inst * v.npe + e]);
    const float* base = v.vsu + (size_t)inst * VSU_K * v.np;
    float acc[3][3][4];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int m = 0; m < 4; ++m) acc[d][j][m] = 0.f;
#pragma unroll
    for (int type = 0; type < 3; ++type) {
        float x[8][6];
#pragma unroll
        for (int l = 0; l < 8; ++l)
#pragma unroll
            for (int c = 0; c < 6; ++c) x[l][c] = base[(size_t)(type * 6 + c) * v.np + node[l]];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int c = cdp_fcomp(d, j);
                float z[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) z[m] = x[cdp_lex(d, m, 0)][c] + x[cdp_lex(d, m, 1)][c];
                cdp_interp2(z);
#pragma unroll
                for (int m = 0; m < 4; ++m) acc[d][j][m] += cdp_w(s, d, m, type) * z[m];
            }
    }
    float f[8][3];
#pragma unroll
    for (int l = 0; l < 8; ++l) f[l][0] = f[l][1] = f[l][2] = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            cdp_interp2(acc[d][j]);
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                f[cdp_lex(d, m, 1)][j] += acc[d][j][m];
                f[cdp_lex(d, m, 0)][j] -= acc[d][j][m];
            }
        }
    const float hh = 0.5f * v.h, scale = hh * hh * hh / v.h;     // w|J| times the 1/h of the derivative
    float o[24];
#pragma unroll
    for (int l = 0; l < 8; ++l)
#pragma unroll
        for (int j = 0; j < 3; ++j) o[cdp_lex_node(l) * 3 + j] = scale * f[l][j];
    float* out = v.feu + (size_t)inst * 24 * v.npe + e;
#pragma unroll
    for (int i = 0; i < 24; ++i) out[(size_t)i * v.npe] = o[i];
    }
}

// Displacement rows of the PML nodes: R = -(fsol + sum of the element slots)
// - Ku u - Gu ubar + c (u - u_{n-1}), du = R / d; u_{n+1} = u + du and
// ubar += dt (u + du/2) as pairs; the stress rows' inputs.  One thread per
// PML node, looping over the instances.
__global__ void __launch_bounds__(256, 4) k_cdp_uu(CdpView v) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)v.np) return;
    const int p = (int)gid;
    int slots[8];
#pragma unroll
    for (int s2 = 0; s2 < 8; ++s2) slots[s2] = v.ninv[(size_t)p * 8 + s2];
    const long long np0 = v.npad[p];
#pragma unroll 1
    for (int inst = 0; inst < v.ninst; ++inst) {
        const long long pad = (long long)inst * v.per + np0;
        float f[3] = {v.fsol[pad], v.fsol[pad + 1], v.fsol[pad + 2]};
        const size_t fb = (size_t)inst * 24 * v.npe;
#pragma unroll
        for (int s2 = 0; s2 < 8; ++s2) {
            if (slots[s2] < 0) break;
            const float* fe = v.feu + fb + (size_t)(slots[s2] & 7) * 3 * v.npe + (slots[s2] >> 3);
            f[0] += fe[0]; f[1] += fe[v.npe]; f[2] += fe[2 * (size_t)v.npe];
        }
        const float* c6 = v.uc + ((size_t)inst * v.np + p) * 6;
        const float cc = c6[3], Ku = c6[4], Gu = c6[5];
        const size_t ib = ((size_t)inst * v.np + p) * 3;
        float vi[9];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float uh = v.uh[pad + c], ul = v.ul[pad + c], ph = v.uph[pad + c], pl = v.upl[pad + c];
            const float bh = v.ubh[ib + c], bl = v.ubl[ib + c];
            const float u = uh + ul;
            const float R = -f[c] - Ku * u - Gu * bh + cc * ((uh - ph) + (ul - pl));
            const float du = c6[c] * R;
            float nh, nl;
            df_add(uh, ul, du, 0.f, nh, nl);
            v.uph[pad + c] = nh;
            v.upl[pad + c] = nl;
            const float inc = v.dt * (u + 0.5f * du);
            float bh2, bl2;
            df_add(bh, bl, inc, 0.f, bh2, bl2);
            v.ubh[ib + c] = bh2;
            v.ubl[ib + c] = bl2;
            vi[c] = du / v.dt;
            vi[3 + c] = u + 0.5f * du;
            vi[6 + c] = bh + 0.5f * inc;
        }
        float* o = v.vin + (size_t)inst * VIN_K * v.np + p;
#pragma unroll
        for (int k = 0; k < VIN_K; ++k) o[(size_t)k * v.np] = vi[k];
    }
}

// Coupling forces of the PML elements on the stress rows:
// C_Su udot + K_Su umid + G_Su ubar_half = w |J| sum_q N_j(q) E(q), E the
// stretched strain: E_(d,c) = C_d d(udot_c)/dx_d + K_d d(umid_c)/dx_d +
// G_d d(ubar_c)/dx_d, symmetric pairs added.  One thread per element; the
// derivative along d is a difference along d, E_(d,c) does not depend on the
// abscissa along d, and the shape functions along d sum to one over its two
// points, so each term is a 2 x 2 x 2 map over the two other axes whose
// result is the same at both nodes along d.
template <int NT>
__global__ void __launch_bounds__(NT, 512 / NT) k_cdp_fs(CdpView v) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)v.npe) return;
    const int e = (int)gid;
    int node[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) node[l] = v.enode[(size_t)e * 8 + cdp_lex_node(l)];
    float4 t[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) t[d] = reinterpret_cast<const float4*>(v.estr + (size_t)e * 12)[d];
#pragma unroll 1
    for (int inst = 0; inst < v.ninst; ++inst) {
    const CdpStretch s = cdp_stretch(t, v.eb0[(size_t)inst * v.npe + e]);
    const float* base = v.vin + (size_t)inst * VIN_K * v.np;
    float acc[3][3][4];                 // [d][c][m]
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int m = 0; m < 4; ++m) acc[d][c][m] = 0.f;
#pragma unroll
    for (int type = 0; type < 3; ++type) {
        float x[8][3];
#pragma unroll
        for (int l = 0; l < 8; ++l)
#pragma unroll
            for (int c = 0; c < 3; ++c) x[l][c] = base[(size_t)(type * 3 + c) * v.np + node[l]];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float z[4];
#pragma unroll
                for (int m = 0; m < 4; ++m) z[m] = x[cdp_lex(d, m, 1)][c] - x[cdp_lex(d, m, 0)][c];
                cdp_interp2(z);
#pragma unroll
                for (int m = 0; m < 4; ++m) acc[d][c][m] += cdp_w(s, d, m, type) * z[m];
            }
    }
    float r[8][6];
#pragma unroll
    for (int l = 0; l < 8; ++l)
#pragma unroll
        for (int k = 0; k < 6; ++k) r[l][k] = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int k = cdp_scomp(d, c);
            cdp_interp2(acc[d][c]);
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                r[cdp_lex(d, m, 0)][k] += acc[d][c][m];
                r[cdp_lex(d, m, 1)][k] += acc[d][c][m];
            }
        }
    const float hh = 0.5f * v.h, scale = hh * hh * hh / v.h;
    float o[48];
#pragma unroll
    for (int l = 0; l < 8; ++l)
#pragma unroll
        for (int k = 0; k < 6; ++k) o[cdp_lex_node(l) * 6 + k] = scale * r[l][k];
    float* out = v.fes + (size_t)inst * 48 * v.npe + e;
#pragma unroll
    for (int i = 0; i < 48; ++i) out[(size_t)i * v.npe] = o[i];
    }
}

// y = M x for a stress block of isotropic structure: diagonal d and
// off-diagonal o on the normal components (xx yy zz), s on the shear ones.
__device__ __forceinline__ void cdp_block(float d, float o, float s, const float x[6], float y[6]) {
    y[0] = d * x[0] + o * (x[1] + x[2]);
    y[1] = d * x[1] + o * (x[0] + x[2]);
    y[2] = d * x[2] + o * (x[0] + x[1]);
    y[3] = s * x[3];
    y[4] = s * x[4];
    y[5] = s * x[5];
}

// Stress rows of the PML nodes: R = -Fs - KG S - Gs Sbar + A (S - S_prev),
// dS = Dinv R; S_next = S + dS and Sbar += dt S as pairs; and the next
// step's displacement-row inputs (sdot = dS/dt, smid = S + dS/2, Sbar).  One
// thread per PML node, looping over the instances.
__global__ void __launch_bounds__(256, 4) k_cdp_su(CdpView v) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)v.np) return;
    const int p = (int)gid;
    int slots[8];
#pragma unroll
    for (int s2 = 0; s2 < 8; ++s2) slots[s2] = v.ninv[(size_t)p * 8 + s2];
#pragma unroll 1
    for (int inst = 0; inst < v.ninst; ++inst) {
        float F[6] = {0, 0, 0, 0, 0, 0};
        const size_t fb = (size_t)inst * 48 * v.npe;
#pragma unroll
        for (int s2 = 0; s2 < 8; ++s2) {
            if (slots[s2] < 0) break;
            const float* fe = v.fes + fb + (size_t)(slots[s2] & 7) * 6 * v.npe + (slots[s2] >> 3);
#pragma unroll
            for (int c = 0; c < 6; ++c) F[c] += fe[(size_t)c * v.npe];
        }
        const size_t b = ((size_t)inst * v.np + p) * 6;
        float sc[6], ds[6], sb[6], ch[6], cl[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            ch[c] = v.sh[b + c]; cl[c] = v.sl[b + c];
            const float ph = v.sph[b + c], pl = v.spl[b + c];
            sc[c] = ch[c] + cl[c];
            ds[c] = (ch[c] - ph) + (cl[c] - pl);
            sb[c] = v.sbh[b + c];
        }
        const float4* K4 = reinterpret_cast<const float4*>(v.scs + ((size_t)inst * v.np + p) * SCS_ROW);
        const float4 k0 = K4[0], k1 = K4[1], k2 = K4[2];
        float t1[6], t2[6], t3[6], R[6], dS[6];
        cdp_block(k1.z, k1.w, k2.x, sc, t1);      // KG S
        cdp_block(k2.y, k2.z, k2.w, sb, t2);      // Gs Sbar
        cdp_block(k0.w, k1.x, k1.y, ds, t3);      // A (S - S_prev)
#pragma unroll
        for (int c = 0; c < 6; ++c) R[c] = -F[c] - t1[c] - t2[c] + t3[c];
        cdp_block(k0.x, k0.y, k0.z, R, dS);       // Dinv R
        float nx[18];
        const float idt = 1.0f / v.dt;
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            float nh, nl;
            df_add(ch[c], cl[c], dS[c], 0.f, nh, nl);
            v.sph[b + c] = nh;
            v.spl[b + c] = nl;
            float bh, bl;
            df_add(sb[c], v.sbl[b + c], v.dt * sc[c], 0.f, bh, bl);
            v.sbh[b + c] = bh;
            v.sbl[b + c] = bl;
            nx[c] = dS[c] * idt;
            nx[6 + c] = sc[c] + 0.5f * dS[c];
            nx[12 + c] = bh + bl;
        }
        float* o = v.vsu + (size_t)inst * VSU_K * v.np + p;
#pragma unroll
        for (int k = 0; k < VSU_K; ++k) o[(size_t)k * v.np] = nx[k];
    }
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
    double hgrid = 0;                    // element side (uniform cubes)
    bool b_exact = false;                // the B image is exact in TF32 (see the image's construction)
    float kscale = 1.0f;
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
    std::vector<long long> pad_index;    // total dof -> padded position (displacement dofs), or
                                         // -(1 + p*6 + c) for stress dof c of PML node p; one instance
    long long* d_hmap = nullptr;         // history map (k_cdx_hist), hist_n entries
    long long hist_n = 0;                // history entries per step: the instances' total dofs
    int32_t* d_tiles = nullptr;          // ensembles: compact tile -> tile of the full enumeration
    // ensembles of uneven grids: each instance is embedded in the bounding grid;
    // own2emb[b][t] is the embedded total dof of the instance's own dof t
    std::vector<std::vector<long long>> own2emb;
    std::vector<long long> own_ntotal;   // total dofs of each instance in its own numbering
    // PML band (np = 0 without PML elements)
    int np = 0, npe = 0;
    float* fsol = nullptr;
    float *sh[2] = {nullptr, nullptr}, *sl[2] = {nullptr, nullptr};
    float *sbh = nullptr, *sbl = nullptr, *ubh = nullptr, *ubl = nullptr;
    float *vin = nullptr, *vsu = nullptr, *feu = nullptr, *fes = nullptr, *uc = nullptr, *scs = nullptr, *estr = nullptr, *eb0 = nullptr;
    int32_t *enode = nullptr, *ninv = nullptr;
    long long* npad = nullptr;
    int cur = 0;                         // index of u_n in uh/ul
    int64_t launches = 0, launches_last = 0;
    bool va_valid = false;
    // history: two device chunks, filled on `stream`, drained on `copy_stream`
    double* hist[2] = {nullptr, nullptr};
    int hist_cap = 0;                    // steps per chunk
    cudaStream_t copy_stream = nullptr;
    // the PML band runs on its own stream: its stress rows and the next step's
    // element forces overlap the next tensor-core step, which needs only the
    // band's displacement update (ev_uu).  The band's chain of kernels is the
    // longer one, so its stream has the higher priority.
    cudaStream_t bstream = nullptr;
    cudaEvent_t ev_c = nullptr, ev_uu = nullptr, ev_band = nullptr;
    cudaEvent_t ev_hist[2] = {nullptr, nullptr};   // history row of the last even / odd step (band stream)
    // schedule (svl_cdx_set_schedule / svl_cdx_tune): tile order of the fused
    // kernel, block size of the band's element kernels, band stream priority
    std::vector<int32_t> tiles_base;     // the scheduled tiles in natural order (full ids)
    // with a PML band: tiles whose owned nodes and halo hold no PML node
    // ("far" tiles) come first in d_tiles; they step without waiting for the
    // band's displacement update of the previous step
    std::vector<char> tile_near;         // [ntz][nty][ntx] 1: a PML node in the tile or its halo
    int ntiles_far = 0;
    int tile_order = 0, band_threads = 128, band_hi = 1;
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
        if (bstream) cudaStreamSynchronize(bstream);
        if (bstream) cudaStreamDestroy(bstream);
        for (cudaEvent_t e : {ev_c, ev_uu, ev_band, ev_hist[0], ev_hist[1]})
            if (e) cudaEventDestroy(e);
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
    if (m.has_pml())
        for (int e = 0; e < m.nelem; ++e)
            if (m.epml[e] && m.mtype[m.emat[e]] != SVL_MAT_ELASTIC3DLINEAR) { set_error("instance %d: PML element %d needs Elastic3DLinear", inst, e); return SVL_ERR_UNSUPPORTED; }
    if (!m.ray.empty()) { set_error("instance %d: Rayleigh damping is served by the general path (svl_cd_create)", inst); return SVL_ERR_UNSUPPORTED; }
    for (int k = 0; k < m.nmat; ++k)
        if (m.mtype[k] != SVL_MAT_ELASTIC3DLINEAR) { set_error("instance %d: only Elastic3DLinear on the structured path", inst); return SVL_ERR_UNSUPPORTED; }
    // node coordinates on the grid, PlainScheme total dofs node by node (3, or 9
    // at the nodes of PML elements), generator connectivity
    long long off = 0;
    for (long long n = 0; n < nn; ++n) {
        const int i = (int)(n % (nx + 1)), j = (int)((n / (nx + 1)) % (ny + 1)), k = (int)(n / ((long long)(nx + 1) * (ny + 1)));
        const double X[3] = {g->origin[0] + i * g->h[0], g->origin[1] + j * g->h[1], g->origin[2] + k * g->h[2]};
        for (int c = 0; c < 3; ++c)
            if (std::fabs(m.X[n * 3 + c] - X[c]) > 1e-9 * (1.0 + std::fabs(X[c]))) { set_error("instance %d: node %lld is off the grid", inst, n); return SVL_ERR_INVALID; }
        const int nd = m.nndof[n];
        if (nd != 3 && nd != 9) { set_error("instance %d: node %lld has %d dofs", inst, n, nd); return SVL_ERR_INVALID; }
        for (int c = 0; c < nd; ++c)
            if (m.tdof_all[(size_t)n * m.dstride + c] != off + c) { set_error("instance %d: total dofs are not in PlainScheme grid order", inst); return SVL_ERR_INVALID; }
        off += nd;
    }
    if (off != m.ntotal) { set_error("instance %d: total dof count mismatch", inst); return SVL_ERR_INVALID; }
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
// Device pairs of instance `inst` -> FP64 total-dof vector: displacement dofs
// from (dh, dl) (padded layout), stress dofs of PML nodes from (sh, sl) or 0.
static int fetch_pair(svl_cdx* h, const float* dh, const float* dl, int inst, double* out,
                      const float* sh = nullptr, const float* sl = nullptr) {
    const size_t per = h->nstate / h->ninst, n6 = (size_t)h->np * 6;
    std::vector<float> hi(per), lo(per), shi(n6, 0.f), slo(n6, 0.f);
    CUDA_TRY(cudaMemcpyAsync(hi.data(), dh + (size_t)inst * per, per * 4, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaMemcpyAsync(lo.data(), dl + (size_t)inst * per, per * 4, cudaMemcpyDeviceToHost, h->stream));
    if (sh && n6 > 0) {
        CUDA_TRY(cudaMemcpyAsync(shi.data(), sh + (size_t)inst * n6, n6 * 4, cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(cudaMemcpyAsync(slo.data(), sl + (size_t)inst * n6, n6 * 4, cudaMemcpyDeviceToHost, h->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    const bool emb = !h->own2emb.empty();
    for (long long t = 0; t < h->own_ntotal[inst]; ++t) {
        const long long p = h->pad_index[emb ? h->own2emb[inst][t] : t];
        out[t] = p >= 0 ? (double)hi[p] + (double)lo[p] : (double)shi[-p - 1] + (double)slo[-p - 1];
    }
    return SVL_OK;
}

extern "C" {

// Creates the handle for ninst instances on grid g.  Ensembles of uneven
// grids come embedded in their bounding grid: ext [ninst][3] gives each
// instance's own node extents (the tiles beyond them are not scheduled) and
// emb its own-to-embedded dof maps; both null for instances of one grid.
static int upload_tile_order(svl_cdx* h, int order);

static int cdx_create_impl(const svl_grid_spec* g, int32_t ninst, const svl_model_desc* models,
                           const svl_load_desc* loads, const svl_cd_opts* opts, svl_cdx** out, const int32_t* ext,
                           const std::vector<std::vector<long long>>* emb) {
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
    h->ntotal = 0;                                    // from the first instance's numbering
    h->pitch = (nxn * 3 + 3) / 4 * 4;
    const long long per = (long long)h->pitch * nyn * nzn;
    h->nstate = per * ninst;
    h->ntx = (nxn + TX - 1) / TX; h->nty = (nyn + TY - 1) / TY; h->ntz = (nzn + TZ - 1) / TZ;
    const long long ntiles = (long long)h->ntx * h->nty * h->ntz * ninst;
    if (ntiles > INT32_MAX || h->nstate > ((long long)1 << 40)) { set_error("grid too large"); return fail(SVL_ERR_INVALID); }
    h->ntiles = (int)ntiles;
    std::vector<int32_t> tiles;                      // ensembles: the tiles that meet an instance's own nodes
    if (ext) {
        for (int b = 0; b < ninst; ++b)
            for (int tz = 0; tz < (ext[3 * b + 2] + TZ - 1) / TZ; ++tz)
                for (int ty = 0; ty < (ext[3 * b + 1] + TY - 1) / TY; ++ty)
                    for (int tx = 0; tx < (ext[3 * b] + TX - 1) / TX; ++tx) {
                        tiles.push_back((int32_t)((((long long)b * h->ntz + tz) * h->nty + ty) * h->ntx + tx));
                    }
        h->ntiles = (int)tiles.size();
    }
    h->dt = opts->dt;
    h->hgrid = g->h[0];
    {
        int lo_pri = 0, hi_pri = 0;
        if (cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri) != cudaSuccess ||
            cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, lo_pri) != cudaSuccess ||
            cudaStreamCreateWithPriority(&h->bstream, cudaStreamNonBlocking, hi_pri) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_c, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_uu, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_band, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_hist[0], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&h->ev_hist[1], cudaEventDisableTiming) != cudaSuccess) {
            set_error("cudaStreamCreate failed"); return fail(SVL_ERR_CUDA);
        }
    }
    // PML band tables (np = 0 without PML elements)
    std::vector<int32_t> pidx;                       // node -> PML node index or -1
    std::vector<int32_t> t2node;                     // total dof -> node (instance 0 numbering)
    std::vector<int32_t> enode, ninv;
    std::vector<long long> npad;
    std::vector<float> estr, eb0, uc, scs;
    std::vector<int> pelem;                          // PML elements in element order
    std::vector<double> par0;                        // instance 0's PML parameters

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
    // the per-instance host work (model, checks, lumped masses, the explicit
    // PML scheme's tables) runs on one thread per instance
    std::vector<HostModel> hms(ninst);
    std::vector<std::vector<double>> masses(ninst);
    std::vector<ExplicitPmlTables> ptabs(ninst);
    std::vector<int> pst(ninst, SVL_OK);
    {
        auto work = [&](int b) {
            HostModel& m = hms[b];
            if (!model_from_desc(&models[b], m)) { pst[b] = SVL_ERR_INVALID; return; }
            if ((pst[b] = cdx_check_instance(g, m, b))) return;
            lumped_mass_diag(m, opts->mtol, masses[b]);
            if (m.has_pml()) {
                LoadTables lt;
                if ((pst[b] = build_load_tables(m, loads ? &loads[b] : nullptr, lt))) return;
                pst[b] = explicit_pml_tables(m, opts->dt, opts->mtol, lt, ptabs[b]);
            }
        };
        std::vector<std::thread> th;
        for (int b = 0; b < ninst; ++b) th.emplace_back(work, b);
        for (auto& t : th) t.join();
    }
    for (int b = 0; b < ninst; ++b) {
        if (pst[b]) return fail(pst[b]);
        HostModel& m = hms[b];
        if (b == 0) {
            // numbering maps and the PML band layout, shared by every instance
            h->ntotal = m.ntotal;
            h->pad_index.assign(h->ntotal, 0);
            t2node.assign(h->ntotal, -1);
            pidx.assign(h->nn, -1);
            if (m.has_pml()) {
                for (int e = 0; e < m.nelem; ++e)
                    if (m.epml[e]) {
                        pelem.push_back(e);
                        for (int a = 0; a < 8; ++a) pidx[m.conn[(size_t)e * 8 + a]] = 0;
                    }
                for (long long n = 0; n < h->nn; ++n)
                    if (pidx[n] == 0) { pidx[n] = h->np; npad.push_back(0); ++h->np; }
                    else pidx[n] = -1;
                // pidx was marked 0 for PML nodes: rebuild in node order
            }
            for (long long n = 0; n < h->nn; ++n) {
                const long long x = n % nxn, y = (n / nxn) % nyn, z = n / ((long long)nxn * nyn);
                for (int c = 0; c < m.nndof[n]; ++c) {
                    const long long t = m.tdof_all[(size_t)n * m.dstride + c];
                    t2node[t] = (int32_t)n;
                    if (c < 3) h->pad_index[t] = (z * nyn + y) * h->pitch + x * 3 + c;
                    else h->pad_index[t] = -(1 + (long long)pidx[n] * 6 + (c - 3));
                }
                if (pidx[n] >= 0) {
                    npad[pidx[n]] = (z * nyn + y) * h->pitch + x * 3;
                    if (m.nndof[n] != 9) { set_error("PML node %lld has %d dofs", n, m.nndof[n]); return fail(SVL_ERR_INVALID); }
                } else if (m.nndof[n] != 3) {
                    set_error("node %lld of no PML element has %d dofs", n, m.nndof[n]); return fail(SVL_ERR_INVALID);
                }
            }
            h->npe = (int)pelem.size();
            if (h->npe > 0) {
                par0.assign(m.pml_par.begin(), m.pml_par.end());
                enode.resize((size_t)h->npe * 8);
                estr.resize((size_t)h->npe * 12);
                ninv.assign((size_t)h->np * 8, -1);
                std::vector<int> fill(h->np, 0);
                for (int i = 0; i < h->npe; ++i) {
                    const int e = pelem[i];
                    const double* pp = &m.pml_par[(size_t)e * 9];
                    for (int a = 0; a < 8; ++a) {
                        const int pn = pidx[m.conn[(size_t)e * 8 + a]];
                        enode[(size_t)i * 8 + a] = pn;
                        if (fill[pn] >= 8) { set_error("PML node %d in more than 8 elements", pn); return fail(SVL_ERR_INVALID); }
                        ninv[(size_t)pn * 8 + fill[pn]++] = i * 8 + a;
                    }
                    // stretching at the two Gauss abscissae of every axis
                    // (PML3DHexa8.cpp:952-996): a = 1 + a0 r, b = b0 r with
                    // r = ((x - x0) n / L)^m; b0 depends on the material (per instance)
                    const int n1 = m.conn[(size_t)e * 8];
                    const double pm = pp[0], L = pp[1], R = pp[2];
                    const double a0 = (pm + 1.0) * (L / 10.0) / 2.0 / L * std::log(1.0 / R);
                    for (int d = 0; d < 3; ++d)
                        for (int sgn = 0; sgn < 2; ++sgn) {
                            const double xi = sgn ? kGaussAbscissa : -kGaussAbscissa;
                            const double xg = m.X[(size_t)n1 * 3 + d] + 0.5 * g->h[d] * (1.0 + xi);
                            const double r = std::pow((xg - pp[3 + d]) * pp[6 + d] / L, pm);
                            estr[(size_t)i * 12 + 4 * d + sgn] = (float)(1.0 + a0 * r);
                            estr[(size_t)i * 12 + 4 * d + 2 + sgn] = (float)r;
                        }
                }
            }
        } else {
            if (m.ntotal != h->ntotal) { set_error("instance %d: dof count differs from instance 0", b); return fail(SVL_ERR_INVALID); }
            for (int e = 0; e < m.nelem; ++e) {
                const bool pe0 = !pelem.empty() && std::binary_search(pelem.begin(), pelem.end(), e);
                if ((m.has_pml() && m.epml[e]) != pe0) { set_error("instance %d: PML layout differs from instance 0", b); return fail(SVL_ERR_INVALID); }
                if (pe0)
                    for (int j = 0; j < 9; ++j)
                        if (m.pml_par[(size_t)e * 9 + j] != par0[(size_t)e * 9 + j]) { set_error("instance %d: PML parameters differ from instance 0", b); return fail(SVL_ERR_INVALID); }
            }
        }
        if (h->np > 0 && !(g->h[1] == g->h[0] && g->h[2] == g->h[0])) {
            set_error("the PML band of the structured path needs cubic elements"); return fail(SVL_ERR_UNSUPPORTED);
        }
        if (h->np > 0) {
            // explicit scheme tables of this instance (lumped blocks, solves)
            const ExplicitPmlTables& T = ptabs[b];
            const double dt = opts->dt;
            static const int pk[9][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {1, 2}, {0, 2}, {3, 3}, {4, 4}, {5, 5}};
            for (long long n = 0; n < h->nn; ++n) {
                const int pn = pidx[n];
                if (pn < 0) continue;
                const int t0 = m.tdof_all[(size_t)n * m.dstride];
                float u6[6];
                for (int c = 0; c < 3; ++c) {
                    const int f = m.fdof_all[(size_t)n * m.dstride + c];
                    u6[c] = f >= 0 ? (float)T.kinv[f] : 0.f;
                    if (T.Mu[t0 + c] != T.Mu[t0] || T.Ku[t0 + c] != T.Ku[t0] || T.Gu[t0 + c] != T.Gu[t0] || T.Cu[t0 + c] != T.Cu[t0]) {
                        set_error("instance %d: PML node %lld has unequal lumped blocks per component", b, n); return fail(SVL_ERR_UNSUPPORTED);
                    }
                    if (f < -1) { set_error("instance %d: constraints are not supported on the structured path", b); return fail(SVL_ERR_UNSUPPORTED); }
                }
                u6[3] = (float)(1.0 / dt / dt * T.Mu[t0] - 1.0 / 2.0 / dt * T.Cu[t0]);
                u6[4] = (float)T.Ku[t0];
                u6[5] = (float)T.Gu[t0];
                uc.insert(uc.end(), u6, u6 + 6);
                const int sn = T.snode_of[n];
                const double* Ms = &T.Ms[(size_t)sn * 36];
                const double* Cs = &T.Cs[(size_t)sn * 36];
                const double* Ks = &T.Ks[(size_t)sn * 36];
                const double* Gs = &T.Gs[(size_t)sn * 36];
                const double* Di = &T.Dinv[(size_t)sn * 36];
                double blk[36];
                for (int k2 = 0; k2 < 9; ++k2) {
                    const int i = pk[k2][0] * 6 + pk[k2][1];
                    blk[k2] = Di[i];
                    blk[9 + k2] = Ms[i] / dt / dt - Cs[i] / 2.0 / dt;
                    blk[18 + k2] = Ks[i] + dt / 2.0 * Gs[i];
                    blk[27 + k2] = Gs[i];
                }
                // isotropic materials give every block the form d I + o (1 1^T - I) on the
                // normal components and s I on the shear ones: three numbers per block
                for (int kb = 0; kb < 4; ++kb) {
                    const double* B = blk + 9 * kb;
                    const double sc2 = std::max(std::fabs(B[0]), std::fabs(B[3])), tol = 1e-10;
                    if (std::fabs(B[1] - B[0]) > tol * sc2 || std::fabs(B[2] - B[0]) > tol * sc2 ||
                        std::fabs(B[4] - B[3]) > tol * sc2 || std::fabs(B[5] - B[3]) > tol * sc2 ||
                        std::fabs(B[7] - B[6]) > tol * std::fabs(B[6]) || std::fabs(B[8] - B[6]) > tol * std::fabs(B[6])) {
                        set_error("instance %d: PML node %lld has a stress block without isotropic structure", b, n);
                        return fail(SVL_ERR_UNSUPPORTED);
                    }
                    scs.push_back((float)B[0]);
                    scs.push_back((float)B[3]);
                    scs.push_back((float)B[6]);
                }
            }
            for (int i = 0; i < h->npe; ++i) {
                const double* pr = m.param(pelem[i]);
                const double* pp = &m.pml_par[(size_t)pelem[i] * 9];
                const double E = pr[0], nu = pr[1], rho = pr[2];
                const double mu = E / 2.0 / (1 + nu), lambda = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu);
                const double Vp = std::sqrt((lambda + 2.0 * mu) / rho);
                eb0.push_back((float)((pp[0] + 1.0) * Vp / 2.0 / pp[1] * std::log(1.0 / pp[2])));
            }
        }
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
            const bool pml_e = m.has_pml() && m.epml[e];      // PML elements: no elastic force here
            lam[li] = pml_e ? 0.f : (float)(E * nu / (1.0 - 2.0 * nu) / (1.0 + nu));
            mu[li] = pml_e ? 0.f : (float)(E / (2.0 * (1.0 + nu)));
        }
        const std::vector<double>& M = masses[b];
        for (long long n = 0; n < h->nn; ++n)
            for (int c = 0; c < 3; ++c) {
                const long long t = m.tdof_all[(size_t)n * m.dstride + c];
                const int f = m.fdof_all[(size_t)n * m.dstride + c];
                float cd;
                if (pidx[n] >= 0) cd = -1.0f;                 // updated by the PML kernels
                else {
                    const bool fixed = f < 0;
                    if (!fixed && !(M[t] > 0)) { set_error("instance %d: free dof %lld has no mass", b, t); return fail(SVL_ERR_INVALID); }
                    cd = fixed ? 0.0f : (float)(dt2 / M[t]);
                }
                cdof[(size_t)b * per + h->pad_index[t]] = cd;
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
                if (h->pad_index[L.force_dof[i2]] < 0 || pidx[t2node[L.force_dof[i2]]] >= 0) {
                    set_error("instance %d: load entry %d is on a PML node (not covered on the structured path)", b, i2);
                    return fail(SVL_ERR_UNSUPPORTED);
                }
                fdof.push_back((long long)b * h->ntotal + L.force_dof[i2]);
                fser.push_back(soff + L.force_series[i2]);
                fcoef.push_back(L.force_coef[i2]);
            }
        }
    }
    // B operand image, canonical K-major layout, 96 rows:
    // [K_lambda hi; K_mu hi; K_lambda lo; K_mu lo] (24 rows each).  For a cube
    // of side h every entry of K_lambda and K_mu is an integer times h/72 (up
    // to the rounding of the Gauss abscissa, ~1e-15): the image then holds the
    // integers, exact in TF32, its lo half is zero, the element force takes
    // two products instead of three and lambda, mu are scaled by h/72.
    std::vector<float> bop(B_BYTES / 4, 0.f);
    {
        const double c = 72.0 / h->hgrid;
        bool exact = g->h[1] == g->h[0] && g->h[2] == g->h[0];
        for (int i2 = 0; i2 < 24 * 24 && exact; ++i2)
            for (double kv : {Klam[i2] * c, Kmu[i2] * c})
                exact = exact && std::fabs(kv - std::nearbyint(kv)) <= 1e-9 && std::fabs(kv) <= 1024.0;
        h->b_exact = exact;
        h->kscale = exact ? (float)(h->hgrid / 72.0) : 1.0f;
        if (exact)
            for (int i2 = 0; i2 < 24 * 24; ++i2) { Klam[i2] = std::nearbyint(Klam[i2] * c); Kmu[i2] = std::nearbyint(Kmu[i2] * c); }
    }
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
        const long long b = gdof / h->ntotal, t = gdof % h->ntotal, n = t2node[t];
        const long long x = n % nxn, y = (n / nxn) % nyn, z = n / ((long long)nxn * nyn);
        return (((b * h->ntz + z / TZ) * h->nty + y / TY) * h->ntx + x / TX);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const long long ta = tile_of(fdof[a]), tc = tile_of(fdof[c]);
        return ta < tc || (ta == tc && fdof[a] < fdof[c]);
    });
    std::vector<int> tl_ptr((size_t)ntiles + 1, 0), ld_ptr(1, 0), ld_ser;
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
    for (long long t = 0; t < ntiles; ++t) tl_ptr[t + 1] += tl_ptr[t];

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
    if (ext && (st = h->upload(tiles, &h->d_tiles))) return fail(st);
    if (ext) h->tiles_base = tiles;
    else {
        h->tiles_base.resize((size_t)h->ntiles);
        for (int t = 0; t < h->ntiles; ++t) h->tiles_base[t] = t;
    }
    if (h->np > 0 && !ext) {
        // a tile reads nodes x0-1 .. x0+TX (and the same in y, z): mark the
        // tiles that meet a PML node there (the layout is every instance's)
        h->tile_near.assign((size_t)h->ntx * h->nty * h->ntz, 0);
        for (long long n = 0; n < h->nn; ++n) {
            if (pidx[n] < 0) continue;
            const int x = (int)(n % nxn), y = (int)((n / nxn) % nyn), z = (int)(n / ((long long)nxn * nyn));
            const int tx0 = std::max(0, (x - TX + TX - 1) / TX), tx1 = std::min(h->ntx - 1, (x + 1) / TX);
            const int ty0 = std::max(0, (y - TY + TY - 1) / TY), ty1 = std::min(h->nty - 1, (y + 1) / TY);
            const int tz0 = std::max(0, (z - TZ + TZ - 1) / TZ), tz1 = std::min(h->ntz - 1, (z + 1) / TZ);
            for (int tz = tz0; tz <= tz1; ++tz)
                for (int ty = ty0; ty <= ty1; ++ty)
                    for (int tx = tx0; tx <= tx1; ++tx) h->tile_near[((size_t)tz * h->nty + ty) * h->ntx + tx] = 1;
        }
        if ((st = upload_tile_order(h, 0))) return fail(st);
    }
    // history map: the instances one after the other, each in its own numbering
    {
        if (emb) h->own2emb = *emb;
        const long long sper = (long long)h->np * 6;
        std::vector<long long> hm;
        for (int b = 0; b < ninst; ++b) {
            const long long n = emb ? (long long)(*emb)[b].size() : h->ntotal;
            h->own_ntotal.push_back(n);
            for (long long t = 0; t < n; ++t) {
                const long long p2 = h->pad_index[emb ? (*emb)[b][t] : t];
                hm.push_back(p2 >= 0 ? b * per + p2 : -(1 + b * sper + (-p2 - 1)));
            }
        }
        h->hist_n = (long long)hm.size();
        if ((st = h->upload(hm, &h->d_hmap))) return fail(st);
    }
    if (h->np > 0) {
        const size_t n6 = (size_t)ninst * h->np * 6, n3 = (size_t)ninst * h->np * 3;
        if ((st = h->alloc(ns, &h->fsol)) || (st = h->alloc(n6, &h->sh[0])) || (st = h->alloc(n6, &h->sh[1])) ||
            (st = h->alloc(n6, &h->sl[0])) || (st = h->alloc(n6, &h->sl[1])) || (st = h->alloc(n6, &h->sbh)) ||
            (st = h->alloc(n6, &h->sbl)) || (st = h->alloc(n3, &h->ubh)) || (st = h->alloc(n3, &h->ubl)) ||
            (st = h->alloc((size_t)ninst * h->np * VIN_K, &h->vin)) || (st = h->alloc((size_t)ninst * h->np * VSU_K, &h->vsu)) ||
            (st = h->alloc((size_t)ninst * h->npe * 24, &h->feu)) || (st = h->alloc((size_t)ninst * h->npe * 48, &h->fes)) ||
            (st = h->upload(uc, &h->uc)) || (st = h->upload(scs, &h->scs)) || (st = h->upload(estr, &h->estr)) ||
            (st = h->upload(eb0, &h->eb0)) || (st = h->upload(enode, &h->enode)) || (st = h->upload(ninv, &h->ninv)) ||
            (st = h->upload(npad, &h->npad)))
            return fail(st);
    }
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

int svl_cdx_create(const svl_grid_spec* g, int32_t ninst, const svl_model_desc* models, const svl_load_desc* loads,
                   const svl_cd_opts* opts, svl_cdx** out) {
    return cdx_create_impl(g, ninst, models, loads, opts, out, nullptr, nullptr);
}

// Ensembles of uneven grids: every instance is embedded in the grid that
// bounds them all (same element size): its nodes keep their coordinates
// relative to the grid origin, numbering and restraints; the rest of the
// bounding lattice gets restrained nodes and elements of a material without
// stiffness or mass, so nothing there moves or loads the instance; the fused
// kernel schedules only the tiles that meet an instance's own nodes.
int svl_cdx_create_ensemble(const svl_grid_spec* grids, int32_t ninst, const svl_model_desc* models,
                            const svl_load_desc* loads, const svl_cd_opts* opts, svl_cdx** out) {
    if (!grids || !models || !opts || !out || ninst <= 0) { set_error("NULL argument or ninst <= 0"); return SVL_ERR_INVALID; }
    *out = nullptr;
    svl_grid_spec gb = grids[0];
    for (int b = 0; b < ninst; ++b) {
        const svl_grid_spec& g = grids[b];
        if (g.ndim != 3) { set_error("the structured mixed path is 3D (lin3DHexa8)"); return SVL_ERR_UNSUPPORTED; }
        for (int d = 0; d < 3; ++d) {
            if (g.ne[d] <= 0) { set_error("instance %d: bad grid", b); return SVL_ERR_INVALID; }
            if (std::fabs(g.h[d] - grids[0].h[d]) > 1e-12 * std::fabs(grids[0].h[d])) {
                set_error("instance %d: every instance needs the element size of instance 0", b); return SVL_ERR_UNSUPPORTED;
            }
            gb.ne[d] = std::max(gb.ne[d], g.ne[d]);
        }
    }
    const int NX = gb.ne[0], NY = gb.ne[1], NZ = gb.ne[2];
    const long long nnb = (long long)(NX + 1) * (NY + 1) * (NZ + 1), neb = (long long)NX * NY * NZ;
    struct Emb {
        std::vector<double> X, mpar, nmass, sval, fcoef;
        std::vector<int32_t> tdof, fdof, conn, emat, mtype, sptr, fdofl, fser;
        svl_model_desc md{};
        svl_load_desc ld{};
    };
    std::vector<Emb> E(ninst);
    std::vector<std::vector<long long>> own2emb(ninst);
    std::vector<int32_t> ext(3 * (size_t)ninst);
    for (int b = 0; b < ninst; ++b) {
        HostModel m;
        if (!model_from_desc(&models[b], m)) return SVL_ERR_INVALID;
        int st = cdx_check_instance(&grids[b], m, b);
        if (st) return st;
        if (m.has_pml()) { set_error("instance %d: ensembles of uneven grids are covered without PML layers", b); return SVL_ERR_UNSUPPORTED; }
        const int nx = grids[b].ne[0], ny = grids[b].ne[1], nz = grids[b].ne[2];
        ext[3 * b] = nx + 1; ext[3 * b + 1] = ny + 1; ext[3 * b + 2] = nz + 1;
        Emb& em = E[b];
        em.X.resize((size_t)nnb * 3);
        em.tdof.resize((size_t)nnb * 3);
        em.fdof.assign((size_t)nnb * 3, -1);
        std::vector<long long> node_emb((size_t)m.nnode);
        for (long long n = 0; n < nnb; ++n) {
            const int i = (int)(n % (NX + 1)), j = (int)((n / (NX + 1)) % (NY + 1)), k = (int)(n / ((long long)(NX + 1) * (NY + 1)));
            const double xyz[3] = {i * gb.h[0], j * gb.h[1], k * gb.h[2]};
            for (int c = 0; c < 3; ++c) { em.X[n * 3 + c] = gb.origin[c] + xyz[c]; em.tdof[n * 3 + c] = (int32_t)(n * 3 + c); }
            if (i <= nx && j <= ny && k <= nz) {
                const long long no = ((long long)k * (ny + 1) + j) * (nx + 1) + i;
                node_emb[no] = n;
                for (int c = 0; c < 3; ++c) em.fdof[n * 3 + c] = m.fdof_all[(size_t)no * m.dstride + c];
            }
        }
        own2emb[b].resize((size_t)m.ntotal);
        for (long long no = 0; no < m.nnode; ++no)
            for (int c = 0; c < 3; ++c) own2emb[b][(size_t)m.tdof_all[(size_t)no * m.dstride + c]] = node_emb[no] * 3 + c;
        // elements: the instance's own where they lie, else a material without stiffness or mass
        em.conn.resize((size_t)neb * 8);
        em.emat.resize((size_t)neb);
        em.mtype.assign(m.mtype.begin(), m.mtype.end());
        em.mtype.push_back(SVL_MAT_ELASTIC3DLINEAR);
        em.mpar.assign(m.mpar.begin(), m.mpar.end());
        em.mpar.resize((size_t)(m.nmat + 1) * SVL_MAT_NPARAM, 0.0);
        em.mpar[(size_t)m.nmat * SVL_MAT_NPARAM + 1] = 0.25;       // E = 0, rho = 0
        const long long layer = (long long)(NX + 1) * (NY + 1);
        long long e = 0;
        for (int k = 0; k < NZ; ++k)
            for (int j = 0; j < NY; ++j)
                for (int i = 0; i < NX; ++i, ++e) {
                    const long long n1 = layer * k + (long long)j * (NX + 1) + i;
                    const long long c8[8] = {n1, n1 + 1, n1 + 1 + (NX + 1), n1 + (NX + 1),
                                             n1 + layer, n1 + layer + 1, n1 + layer + 1 + (NX + 1), n1 + layer + (NX + 1)};
                    for (int a = 0; a < 8; ++a) em.conn[e * 8 + a] = (int32_t)c8[a];
                    em.emat[e] = (i < nx && j < ny && k < nz) ? m.emat[((long long)k * ny + j) * nx + i] : m.nmat;
                }
        if (!m.nodemass.empty()) {
            em.nmass.assign((size_t)nnb * 3, 0.0);
            for (long long t = 0; t < m.ntotal; ++t) em.nmass[own2emb[b][t]] = m.nodemass[t];
        }
        svl_model_desc& d = em.md;
        d.ndim = 3; d.nnode = (int32_t)nnb; d.ndof = 3;
        d.coords = em.X.data(); d.totaldof = em.tdof.data(); d.freedof = em.fdof.data();
        d.ntotal = (int32_t)(nnb * 3); d.nfree = m.nfree;
        d.elem_type = SVL_ELEM_LIN3DHEXA8; d.nelem = (int32_t)neb; d.conn = em.conn.data(); d.elem_mat = em.emat.data();
        d.nmat = m.nmat + 1; d.mat_type = em.mtype.data(); d.mat_param = em.mpar.data();
        d.lumped = m.lumped ? 1 : 0;
        d.node_mass = em.nmass.empty() ? nullptr : em.nmass.data();
        // loads on the embedded numbering
        if (loads) {
            const svl_load_desc& L = loads[b];
            em.sptr.assign(L.series_ptr, L.series_ptr + L.nseries + 1);
            em.sval.assign(L.series_val, L.series_val + (L.nseries > 0 ? L.series_ptr[L.nseries] : 0));
            for (int i2 = 0; i2 < L.nforce; ++i2) {
                if (L.force_dof[i2] < 0 || L.force_dof[i2] >= m.ntotal) { set_error("instance %d: load entry %d out of range", b, i2); return SVL_ERR_INVALID; }
                em.fdofl.push_back((int32_t)own2emb[b][L.force_dof[i2]]);
            }
            em.fser.assign(L.force_series, L.force_series + L.nforce);
            em.fcoef.assign(L.force_coef, L.force_coef + L.nforce);
            if (L.nsupport > 0 || L.ndrm > 0) { set_error("instance %d: support motion and domain-reduction loads are served by svl_cd_create", b); return SVL_ERR_UNSUPPORTED; }
            svl_load_desc& l = em.ld;
            l.nseries = L.nseries; l.series_ptr = em.sptr.data(); l.series_val = em.sval.data();
            l.nforce = L.nforce; l.force_dof = em.fdofl.data(); l.force_series = em.fser.data(); l.force_coef = em.fcoef.data();
        }
    }
    std::vector<svl_model_desc> md(ninst);
    std::vector<svl_load_desc> ld(ninst);
    for (int b = 0; b < ninst; ++b) { md[b] = E[b].md; ld[b] = E[b].ld; }
    return cdx_create_impl(&gb, ninst, md.data(), loads ? ld.data() : nullptr, opts, out, ext.data(), &own2emb);
}

int svl_cdx_set_initial(svl_cdx* h, int32_t inst, const double* U0, const double* V0, const double* A0) {
    if (!h || inst < 0 || inst >= h->ninst) { set_error("bad handle or instance"); return SVL_ERR_INVALID; }
    std::vector<double> ew[3];                       // ensembles: the instance's vectors on its embedding
    if (!h->own2emb.empty()) {
        const double* src[3] = {U0, V0, A0};
        for (int w = 0; w < 3; ++w) {
            if (!src[w]) continue;
            ew[w].assign((size_t)h->ntotal, 0.0);
            for (size_t t = 0; t < h->own2emb[inst].size(); ++t) ew[w][h->own2emb[inst][t]] = src[w][t];
        }
        U0 = U0 ? ew[0].data() : nullptr;
        V0 = V0 ? ew[1].data() : nullptr;
        A0 = A0 ? ew[2].data() : nullptr;
    }
    const size_t per = (size_t)(h->nstate / h->ninst);
    std::vector<float> hi(per, 0.f), lo(per, 0.f), phi(per, 0.f), plo(per, 0.f);
    const size_t n6 = (size_t)h->np * 6;
    std::vector<float> shi(n6, 0.f), slo(n6, 0.f), sphi(n6, 0.f), splo(n6, 0.f);
    for (long long t = 0; t < h->ntotal; ++t) {
        const double u = U0 ? U0[t] : 0.0, vv = V0 ? V0[t] : 0.0, a = A0 ? A0[t] : 0.0;
        const double up = u - h->dt * vv + h->dt * h->dt / 2.0 * a;
        const long long p = h->pad_index[t];
        if (p < 0) {                               // stress dof of a PML node
            const size_t k = (size_t)(-p - 1);
            split_pair(u, shi[k], slo[k]);
            split_pair(up, sphi[k], splo[k]);
            continue;
        }
        split_pair(u, hi[p], lo[p]);
        split_pair(up, phi[p], plo[p]);
    }
    const size_t off = (size_t)inst * per;
    CUDA_TRY(cudaMemcpyAsync(h->uh[h->cur] + off, hi.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->ul[h->cur] + off, lo.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->uh[1 - h->cur] + off, phi.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(cudaMemcpyAsync(h->ul[1 - h->cur] + off, plo.data(), per * 4, cudaMemcpyHostToDevice, h->stream));
    if (h->np > 0) {
        const size_t o6 = (size_t)inst * n6;
        CUDA_TRY(cudaMemcpyAsync(h->sh[h->cur] + o6, shi.data(), n6 * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(cudaMemcpyAsync(h->sl[h->cur] + o6, slo.data(), n6 * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(cudaMemcpyAsync(h->sh[1 - h->cur] + o6, sphi.data(), n6 * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(cudaMemcpyAsync(h->sl[1 - h->cur] + o6, splo.data(), n6 * 4, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(cudaMemsetAsync(h->sbh + o6, 0, n6 * 4, h->stream));
        CUDA_TRY(cudaMemsetAsync(h->sbl + o6, 0, n6 * 4, h->stream));
        CUDA_TRY(cudaMemsetAsync(h->ubh + (size_t)inst * h->np * 3, 0, (size_t)h->np * 12, h->stream));
        CUDA_TRY(cudaMemsetAsync(h->ubl + (size_t)inst * h->np * 3, 0, (size_t)h->np * 12, h->stream));
        // the first step's displacement-row inputs: sdot, smid, Sbar = 0
        std::vector<float> vs((size_t)h->np * VSU_K, 0.f);
        for (size_t k = 0; k < n6; ++k) {
            const size_t p = k / 6, c = k % 6;
            const double sc = (double)shi[k] + slo[k], sp = (double)sphi[k] + splo[k];
            vs[c * h->np + p] = (float)((sc - sp) / h->dt);
            vs[(6 + c) * h->np + p] = (float)((sc + sp) / 2.0);
        }
        CUDA_TRY(cudaMemcpyAsync(h->vsu + (size_t)inst * h->np * VSU_K, vs.data(), vs.size() * 4, cudaMemcpyHostToDevice,
                                 h->stream));
    }
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->va_valid = false;
    return SVL_OK;
}

// The PML band's view of the handle for the step from u_n (index cur).
static CdpView cdp_view(svl_cdx* h) {
    CdpView c{};
    c.ninst = h->ninst; c.np = h->np; c.npe = h->npe;
    c.h = (float)h->hgrid; c.dt = (float)h->dt;
    c.per = (long long)(h->nstate / h->ninst);
    c.enode = h->enode; c.estr = h->estr; c.eb0 = h->eb0; c.ninv = h->ninv; c.npad = h->npad;
    c.uc = h->uc; c.scs = h->scs;
    c.uh = h->uh[h->cur]; c.ul = h->ul[h->cur]; c.uph = h->uh[1 - h->cur]; c.upl = h->ul[1 - h->cur];
    c.fsol = h->fsol;
    c.ubh = h->ubh; c.ubl = h->ubl;
    c.sh = h->sh[h->cur]; c.sl = h->sl[h->cur]; c.sph = h->sh[1 - h->cur]; c.spl = h->sl[1 - h->cur];
    c.sbh = h->sbh; c.sbl = h->sbl; c.vin = h->vin; c.vsu = h->vsu; c.feu = h->feu; c.fes = h->fes;
    return c;
}

// One kernel of the band's step: 0 = k_cdp_fu, 1 = k_cdp_uu (displacement
// rows), 2 = k_cdp_fs, 3 = k_cdp_su (stress rows).  One thread per PML element
// or per PML node, each looping over the instances (their tables are read
// once).
static void cdp_launch(svl_cdx* h, const CdpView& c, int which, cudaStream_t st) {
    const int nt = h->band_threads;
    const unsigned be = (unsigned)((h->npe + nt - 1) / nt), bn = (unsigned)((h->np + 255) / 256);
    switch (which) {
        case 0:
            if (nt == 256) k_cdp_fu<256><<<be, 256, 0, st>>>(c);
            else k_cdp_fu<128><<<be, 128, 0, st>>>(c);
            break;
        case 1: k_cdp_uu<<<bn, 256, 0, st>>>(c); break;
        case 2:
            if (nt == 256) k_cdp_fs<256><<<be, 256, 0, st>>>(c);
            else k_cdp_fs<128><<<be, 128, 0, st>>>(c);
            break;
        default: k_cdp_su<<<bn, 256, 0, st>>>(c); break;
    }
    ++h->launches;
}

// Makes the compute stream wait for everything the band stream has queued.
static int cdx_join(svl_cdx* h) {
    if (h->np == 0) return SVL_OK;
    CUDA_TRY(cudaEventRecord(h->ev_band, h->bstream));
    CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_band, 0));
    return SVL_OK;
}

static int cdx_step(svl_cdx* h, int k, bool want_va) {
    CdxView v;
    v.nx = h->nx; v.ny = h->ny; v.nz = h->nz; v.ninst = h->ninst;
    v.pitch = h->pitch; v.ntx = h->ntx; v.nty = h->nty; v.ntz = h->ntz; v.ntiles = h->ntiles; v.tiles = h->d_tiles;
    v.uh_prev = h->uh[1 - h->cur]; v.ul_prev = h->ul[1 - h->cur];
    v.cdof = h->cdof; v.bop = h->bop;
    v.tl_ptr = h->tl_ptr; v.ld_dof = h->ld_dof; v.ld_ptr = h->ld_ptr; v.ld_ser = h->ld_ser; v.ld_coef = h->ld_coef;
    v.s_ptr = h->s_ptr; v.s_val = h->s_val;
    v.k = k;
    v.kscale = h->kscale;
    v.b_exact = h->b_exact ? 1 : 0;
    v.status = h->status;
    v.fsol = h->fsol;
    const size_t ns = (size_t)h->nstate;
    if (want_va) {
        if (h->np > 0) CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_uu, 0));
        CUDA_TRY(cudaMemcpyAsync(h->ph_copy, v.uh_prev, ns * 4, cudaMemcpyDeviceToDevice, h->stream));
        CUDA_TRY(cudaMemcpyAsync(h->pl_copy, v.ul_prev, ns * 4, cudaMemcpyDeviceToDevice, h->stream));
    }
    auto launch = [&](int first, int count) {
        CdxView w = v;
        w.tiles = v.tiles + first;
        w.ntiles = count;
        k_cdx_step<<<std::min(count, h->grid), NTHREADS, SMEM_BYTES, h->stream>>>(
            h->tmap[h->cur], h->tmap_lam, h->tmap_mu, h->own_ul[h->cur], h->own_uh[1 - h->cur], h->own_ul[1 - h->cur],
            h->own_cd, w);
        ++h->launches;
    };
    if (h->np > 0) {
        // far tiles (no PML node in the tile or its halo) do not read what the
        // band's displacement update of the previous step writes: they run
        // while it finishes; the near tiles wait for it (u_n at the PML nodes)
        if (h->ntiles_far > 0) launch(0, h->ntiles_far);
        CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_uu, 0));
        if (h->ntiles > h->ntiles_far) launch(h->ntiles_far, h->ntiles - h->ntiles_far);
    } else {
        k_cdx_step<<<h->grid, NTHREADS, SMEM_BYTES, h->stream>>>(h->tmap[h->cur], h->tmap_lam, h->tmap_mu, h->own_ul[h->cur],
                                                                 h->own_uh[1 - h->cur], h->own_ul[1 - h->cur], h->own_cd, v);
        ++h->launches;
    }
    if (h->np > 0) {
        // the PML band on its stream: element forces on the displacement rows
        // (inputs from the previous step's stress update, in stream order), then,
        // once the tensor-core step has left fsol, the displacement update
        // (ev_uu), then the stress rows, which overlap the next step
        const CdpView c = cdp_view(h);
        CUDA_TRY(cudaEventRecord(h->ev_c, h->stream));
        cdp_launch(h, c, 0, h->bstream);
        CUDA_TRY(cudaStreamWaitEvent(h->bstream, h->ev_c, 0));
        cdp_launch(h, c, 1, h->bstream);
        CUDA_TRY(cudaEventRecord(h->ev_uu, h->bstream));
        cdp_launch(h, c, 2, h->bstream);
        cdp_launch(h, c, 3, h->bstream);
    }
    if (want_va) {
        if (h->np > 0) CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_uu, 0));
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
// With a PML band the history row of a step is written on the band stream,
// right after the step's stress update (k_cdp_su): the next step's kernels do
// not wait for the band to finish.  The row reads u_{n+1} and S^{n+3/2}, which
// step n + 2 overwrites (its tensor-core step on the compute stream, its band
// kernels after the row in band-stream order): step n + 2 waits for the row's
// event.
static int cdx_fill_chunk(svl_cdx* h, int k_first, int s0, int n, int nsteps, int slot) {
    const long long per_step = h->hist_n;
    const bool band = h->np > 0;
    cudaStream_t hs = band ? h->bstream : h->stream;                      // the stream of the history rows
    CUDA_TRY(cudaStreamWaitEvent(hs, h->drained[slot], 0));              // the chunk's previous copy is done
    for (int i = 0; i < n; ++i) {
        const int s = s0 + i;
        if (band) CUDA_TRY(cudaStreamWaitEvent(h->stream, h->ev_hist[s & 1], 0));   // row of step s - 2
        TRY(cdx_step(h, k_first + s, s == nsteps - 1));
        k_cdx_hist<<<(unsigned)((per_step + 255) / 256), 256, 0, hs>>>(
            h->uh[h->cur], h->ul[h->cur], h->sh[h->cur], h->sl[h->cur], h->d_hmap, h->hist[slot] + (size_t)i * per_step,
            per_step);
        ++h->launches;
        if (band) CUDA_TRY(cudaEventRecord(h->ev_hist[s & 1], h->bstream));
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(h->filled[slot], hs));
    return SVL_OK;
}

int svl_cdx_run(svl_cdx* h, int32_t k_first, int32_t nsteps, double* U_hist) {
    if (!h || nsteps < 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    const int64_t l0 = h->launches;
    if (!U_hist) {
        for (int s = 0; s < nsteps; ++s) TRY(cdx_step(h, k_first + s, s == nsteps - 1));
        TRY(cdx_join(h));
    } else if (nsteps > 0) {
        // device-side FP64 conversion into two chunk buffers; the copy of chunk
        // c (on copy_stream) overlaps the computation of chunk c + 1
        const long long per_step = h->hist_n;
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
        TRY(cdx_join(h));                    // later work on the compute stream follows the band's
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
    TRY(cdx_join(h));
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
    if (which < 0 || which > 3) { set_error("which must be 0, 1, 2 or 3"); return SVL_ERR_INVALID; }
    if (which == 0) return fetch_pair(h, h->uh[h->cur], h->ul[h->cur], inst, out, h->sh[h->cur], h->sl[h->cur]);
    if (which == 3) {                          // ubar / Sbar of the PML nodes, 0 elsewhere
        const size_t n3 = (size_t)h->np * 3, n6 = (size_t)h->np * 6;
        std::vector<float> bh(n3), bl(n3), Sh(n6), Sl(n6);
        if (h->np > 0) {
            CUDA_TRY(cudaMemcpyAsync(bh.data(), h->ubh + inst * n3, n3 * 4, cudaMemcpyDeviceToHost, h->stream));
            CUDA_TRY(cudaMemcpyAsync(bl.data(), h->ubl + inst * n3, n3 * 4, cudaMemcpyDeviceToHost, h->stream));
            CUDA_TRY(cudaMemcpyAsync(Sh.data(), h->sbh + inst * n6, n6 * 4, cudaMemcpyDeviceToHost, h->stream));
            CUDA_TRY(cudaMemcpyAsync(Sl.data(), h->sbl + inst * n6, n6 * 4, cudaMemcpyDeviceToHost, h->stream));
            CUDA_TRY(cudaStreamSynchronize(h->stream));
        }
        std::vector<long long> upos(h->nstate / h->ninst, -1);
        std::vector<long long> npd;
        if (h->np > 0) {
            npd.resize(h->np);
            CUDA_TRY(cudaMemcpy(npd.data(), h->npad, (size_t)h->np * 8, cudaMemcpyDeviceToHost));
            for (int p2 = 0; p2 < h->np; ++p2) upos[npd[p2]] = p2;
        }
        const bool emb = !h->own2emb.empty();
        for (long long t = 0; t < h->own_ntotal[inst]; ++t) {
            const long long p = h->pad_index[emb ? h->own2emb[inst][t] : t];
            if (p < 0) { out[t] = (double)Sh[-p - 1] + (double)Sl[-p - 1]; continue; }
            const long long c = (p % h->pitch) % 3;          // rows hold x*3 + c
            const long long pn = upos[p - c];
            out[t] = pn >= 0 ? (double)bh[pn * 3 + c] + (double)bl[pn * 3 + c] : 0.0;
        }
        return SVL_OK;
    }
    if (!h->va_valid) { set_error("V/A are only available after svl_cdx_run"); return SVL_ERR_INVALID; }
    const size_t per = (size_t)(h->nstate / h->ninst);
    std::vector<double> tmp(per);
    CUDA_TRY(cudaMemcpyAsync(tmp.data(), (which == 1 ? h->V : h->A) + (size_t)inst * per, per * 8, cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    const bool emb = !h->own2emb.empty();
    for (long long t = 0; t < h->own_ntotal[inst]; ++t) out[t] = tmp[h->pad_index[emb ? h->own2emb[inst][t] : t]];
    return SVL_OK;
}

int svl_cdx_profile(svl_cdx* h, int32_t k_first, int32_t nsteps, double* ms_kernel) {
    if (!h || !ms_kernel || nsteps < 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    for (int i = 0; i < 5; ++i) ms_kernel[i] = 0.0;
    cudaEvent_t ev[6];
    for (int i = 0; i < 6; ++i) CUDA_TRY(cudaEventCreate(&ev[i]));
    for (int s2 = 0; s2 < nsteps; ++s2) {
        // the same launches as cdx_step, with events between the kernels:
        // 0 fused tensor-core step, 1 k_cdp_fu, 2 k_cdp_uu, 3 k_cdp_fs, 4 k_cdp_su
        CUDA_TRY(cudaEventRecord(ev[0], h->stream));
        const int np = h->np;
        h->np = 0;                                   // tensor-core kernel alone
        int st = cdx_step(h, k_first + s2, false);
        h->np = np;
        if (st) return st;
        h->cur = 1 - h->cur;                         // cdx_step flipped it; the band still belongs to this step
        CUDA_TRY(cudaEventRecord(ev[1], h->stream));
        const CdpView c = cdp_view(h);
        for (int which = 0; which < 4; ++which) {
            if (np > 0) cdp_launch(h, c, which, h->stream);
            CUDA_TRY(cudaEventRecord(ev[2 + which], h->stream));
        }
        CUDA_TRY(cudaGetLastError());
        h->cur = 1 - h->cur;
        CUDA_TRY(cudaEventSynchronize(ev[5]));
        for (int kind = 0; kind < 5; ++kind) {
            float t = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&t, ev[kind], ev[kind + 1]));
            ms_kernel[kind] += t;
        }
    }
    for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
    h->va_valid = false;
    return cdx_status(h);
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

// The scheduled tiles in one of the orders the tuner tries: 0 natural
// (x fastest, then y, z, instance), 1 instances interleaved (tile position
// first), 2 y fastest, 3 2 x 2 x 2 blocks of tiles.
static std::vector<int32_t> tile_schedule(const svl_cdx* h, int order) {
    std::vector<int32_t> t = h->tiles_base;
    auto key = [&](int32_t full) {
        long long r = full;
        const long long tx = r % h->ntx; r /= h->ntx;
        const long long ty = r % h->nty; r /= h->nty;
        const long long tz = r % h->ntz, b = r / h->ntz;
        const long long X = h->ntx, Y = h->nty, Z = h->ntz, B = h->ninst;
        switch (order) {
            case 1: return ((tz * Y + ty) * X + tx) * B + b;
            case 2: return ((b * Z + tz) * X + tx) * Y + ty;
            case 3: return ((((b * Z + tz / 2) * Y + ty / 2) * X + tx / 2) * 2 + tz % 2) * 4 + (ty % 2) * 2 + tx % 2;
            default: return (long long)full;
        }
    };
    std::stable_sort(t.begin(), t.end(), [&](int32_t a, int32_t c) { return key(a) < key(c); });
    return t;
}

// Uploads the tile order: far tiles first (a stable partition, each part in
// the order's sequence) when the handle has a PML band.
static int upload_tile_order(svl_cdx* h, int order) {
    std::vector<int32_t> t = tile_schedule(h, order);
    h->ntiles_far = 0;
    if (!h->tile_near.empty()) {
        const long long per = (long long)h->ntx * h->nty * h->ntz;
        auto far = [&](int32_t full) { return !h->tile_near[(size_t)(full % per)]; };
        std::stable_partition(t.begin(), t.end(), far);
        h->ntiles_far = (int)std::count_if(t.begin(), t.end(), far);
    }
    if (!h->d_tiles) TRY(h->alloc(t.size(), &h->d_tiles));
    CUDA_TRY(cudaMemcpy(h->d_tiles, t.data(), t.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    h->tile_order = order;
    return SVL_OK;
}

int svl_cdx_set_schedule(svl_cdx* h, const int32_t* choice) {
    if (!h || !choice) { set_error("bad argument"); return SVL_ERR_INVALID; }
    if (choice[1] < 0 || choice[1] > 3 || (choice[2] != 128 && choice[2] != 256) || choice[3] < 0 || choice[3] > 1) {
        set_error("schedule out of range"); return SVL_ERR_INVALID;
    }
    TRY(svl_cdx_set_ctas(h, choice[0]));
    CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (h->bstream) CUDA_TRY(cudaStreamSynchronize(h->bstream));
    if (choice[1] != h->tile_order) TRY(upload_tile_order(h, choice[1]));
    h->band_threads = choice[2];
    if (choice[3] != h->band_hi) {
        int lo_pri = 0, hi_pri = 0;
        CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo_pri, &hi_pri));
        CUDA_TRY(cudaStreamDestroy(h->bstream));
        h->bstream = nullptr;
        CUDA_TRY(cudaStreamCreateWithPriority(&h->bstream, cudaStreamNonBlocking, choice[3] ? hi_pri : lo_pri));
        h->band_hi = choice[3];
    }
    return SVL_OK;
}

int svl_cdx_get_schedule(svl_cdx* h, int32_t* choice) {
    if (!h || !choice) { set_error("bad argument"); return SVL_ERR_INVALID; }
    choice[0] = h->grid; choice[1] = h->tile_order; choice[2] = h->band_threads; choice[3] = h->band_hi;
    return SVL_OK;
}

int svl_cdx_tune(svl_cdx* h, int32_t k_first, int32_t nsteps, int32_t* choice, float* ms_best) {
    if (!h || !choice || nsteps <= 0) { set_error("bad argument"); return SVL_ERR_INVALID; }
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // CTA counts from one per SM down to half of the SMs: fewer step CTAs
    // leave whole SMs to the band kernels, which then overlap the step
    std::vector<int> ctas;
    for (int c : {sms, sms - sms / 16, sms - sms / 8, sms - sms / 4, sms - 5 * sms / 16, sms - 3 * sms / 8,
                  sms - 7 * sms / 16, sms / 2}) {
        c = std::max(1, std::min(c, h->ntiles));                  // as svl_cdx_set_ctas clamps it
        if (std::find(ctas.begin(), ctas.end(), c) == ctas.end()) ctas.push_back(c);
    }
    std::vector<int> bt = {128}, bh = {1};
    if (h->np > 0) { bt.push_back(256); bh.push_back(0); }
    struct Trial { float ms; int32_t ch[4]; };
    std::vector<Trial> trials;
    int k = k_first;
    auto timed = [&](const int32_t* ch, int n, float* ms) -> int {
        TRY(svl_cdx_set_schedule(h, ch));
        for (int w = 0; w < 2; ++w) TRY(cdx_step(h, k++, false));   // warm the choice
        TRY(svl_cdx_run_timed(h, k, n, ms));
        k += n;
        return SVL_OK;
    };
    for (int c : ctas)
        for (int o = 0; o < 4; ++o)
            for (int t : bt)
                for (int p : bh) {
                    Trial tr{0.f, {c, o, t, p}};
                    TRY(timed(tr.ch, nsteps, &tr.ms));
                    trials.push_back(tr);
                }
    // the four fastest again over four times the steps: the pick does not
    // rest on one short sample
    std::sort(trials.begin(), trials.end(), [](const Trial& a, const Trial& b) { return a.ms < b.ms; });
    const size_t nre = std::min<size_t>(4, trials.size());
    float best = 0.f;
    int32_t bc[4] = {0, 0, 128, 1};
    for (size_t i = 0; i < nre; ++i) {
        float ms = 0.f;
        TRY(timed(trials[i].ch, 4 * nsteps, &ms));
        if (best == 0.f || ms < best) { best = ms; std::copy(trials[i].ch, trials[i].ch + 4, bc); }
    }
    TRY(svl_cdx_set_schedule(h, bc));
    std::copy(bc, bc + 4, choice);
    if (ms_best) *ms_best = best / (float)(4 * nsteps);
    h->va_valid = false;
    return SVL_OK;
}

int svl_cdx_launch_count(svl_cdx* h, int64_t* launches) {
    if (!h || !launches) { set_error("bad argument"); return SVL_ERR_INVALID; }
    *launches = h->launches_last;
    return SVL_OK;
}

void svl_cdx_destroy(svl_cdx* h) { delete h; }

}  // extern "C"
