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

    // forward of features already in `feat`; keeps activations
    int forward() {
        const int g = nblocks(d.V);
        k_conv<kNnIn, kNnHid, true><<<g, kThreads, 0, stream>>>(feat, W + kLayers[0].off, a0, d, nullptr);
        k_conv<kNnHid, kNnHid, true><<<g, kThreads, 0, stream>>>(a0, W + kLayers[1].off, a1, d, nullptr);
        k_conv<kNnHid, kNnHid, true><<<g, kThreads, 0, stream>>>(a1, W + kLayers[2].off, a2, d, nullptr);
        k_conv<kNnHid, kNnOut, false><<<g, kThreads, 0, stream>>>(a2, W + kLayers[3].off, y, d, nullptr);
        NN_TRY(cudaGetLastError());
        return SVL_OK;
    }

    template <int CIN, int COUT>
    int wgrad(const float* gout, const float* ain, int layer) {
        dim3 grid(nblk_wg, kNnTaps);
        k_wgrad<CIN, COUT><<<grid, kThreads, 0, stream>>>(gout, ain, partial, d);
        const int n = CIN * COUT * kNnTaps;
        k_wgrad_reduce<<<nblocks(n), kThreads, 0, stream>>>(partial, G + kLayers[layer].off, CIN, COUT, nblk_wg);
        NN_TRY(cudaGetLastError());
        return SVL_OK;
    }

    // data gradient through layer `layer` (cout -> cin), gated by the layer input's relu
    template <int CIN, int COUT>
    int dgrad(const float* gout, float* gin, const float* gate, int layer) {
        const int n = CIN * COUT * kNnTaps;
        k_flip<<<nblocks(n), kThreads, 0, stream>>>(W + kLayers[layer].off, Wt, CIN, COUT);
        k_conv<COUT, CIN, false><<<nblocks(d.V), kThreads, 0, stream>>>(gout, Wt, gin, d, gate);
        NN_TRY(cudaGetLastError());
        return SVL_OK;
    }

    // features of pair p, forward, loss into lsum[slot], gradient accumulated into G
    int sample(const float* x, const float* t, float gscale, float* lslot) {
        const int n3 = 3 * d.V;
        k_feat_grid<<<nblocks(n3), kThreads, 0, stream>>>(x, rho, feat, n3);
        if (int st = forward()) return st;
        k_loss<<<kRedBlocks, kThreads, 0, stream>>>(y, x, t, mask, g3, gscale, lpart, n3);
        k_loss_final<<<1, 32, 0, stream>>>(lpart, lslot, kRedBlocks);
        if (int st = wgrad<kNnHid, kNnOut>(g3, a2, 3)) return st;
        if (int st = dgrad<kNnHid, kNnOut>(g3, gA, a2, 3)) return st;
        if (int st = wgrad<kNnHid, kNnHid>(gA, a1, 2)) return st;
        if (int st = dgrad<kNnHid, kNnHid>(gA, gB, a1, 2)) return st;
        if (int st = wgrad<kNnHid, kNnHid>(gB, a0, 1)) return st;
        if (int st = dgrad<kNnHid, kNnHid>(gB, gA, a0, 1)) return st;
        if (int st = wgrad<kNnIn, kNnHid>(gA, feat, 0)) return st;
        return SVL_OK;
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
    NN_TRY(cudaMemsetAsync(nn->feat, 0, sizeof(float) * kNnIn * (size_t)nn->d.V, nn->stream));
    k_feat_free<<<nblocks(nn->nf), kThreads, 0, nn->stream>>>(r, nn->sdinv, nn->rho, nn->gmap, nn->feat, nn->nf, n3);
    if (int st = nn->forward()) return st;
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

int nn_train(NnPrecond* nn, int iters, int batch, float lr, uint64_t seed, float* loss) {
    const int np = (int)nn->X.size();
    if (np == 0 || iters <= 0 || batch <= 0) { set_error("nothing to train on"); return SVL_ERR_INVALID; }
    if (iters > (1 << 16)) { set_error("at most 65536 training iterations"); return SVL_ERR_INVALID; }
    NN_TRY(cudaMemsetAsync(nn->am, 0, sizeof(float) * kNnWeights, nn->stream));
    NN_TRY(cudaMemsetAsync(nn->av, 0, sizeof(float) * kNnWeights, nn->stream));
    NN_TRY(cudaMemsetAsync(nn->lsum, 0, sizeof(float) * iters, nn->stream));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    uint64_t s = seed ^ 0xD1B54A32D192ED03ull;
    for (int it = 0; it < iters; ++it) {
        NN_TRY(cudaMemsetAsync(nn->G, 0, sizeof(float) * kNnWeights, nn->stream));
        for (int b = 0; b < batch; ++b) {
            s = s * 6364136223846793005ull + 1442695040888963407ull;
            const int p = (int)((s >> 33) % (uint64_t)np);
            if (int st = nn->sample(nn->X[p], nn->Y[p], 1.f / batch, nn->lsum + it)) return st;
        }
        const float frac = (float)it / iters;
        const float lr_it = lr * (frac < 0.6f ? 1.f : (frac < 0.85f ? 0.25f : 0.05f));
        const double c1 = 1.0 - std::pow((double)b1, it + 1), c2 = 1.0 - std::pow((double)b2, it + 1);
        const float lr_t = (float)(lr_it * std::sqrt(c2) / c1);
        k_adam<<<nblocks(kNnWeights), kThreads, 0, nn->stream>>>(nn->W, nn->G, nn->am, nn->av, kNnWeights, lr_t, b1, b2, eps);
        NN_TRY(cudaGetLastError());
    }
    std::vector<float> lh(iters);
    NN_TRY(cudaMemcpyAsync(lh.data(), nn->lsum, sizeof(float) * iters, cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    const int tail = std::max(1, iters / 10);
    double acc = 0.0;
    for (int i = iters - tail; i < iters; ++i) acc += lh[i];
    if (loss) *loss = (float)(acc / tail / batch);
    if (!std::isfinite(acc)) { set_error("training diverged"); return SVL_ERR_NONFINITE; }
    return SVL_OK;
}

int nn_set_weights(NnPrecond* nn, const float* w) {
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

int nn_get_grids(NnPrecond* nn, float* rho, float* mask) {
    const size_t n3 = 3 * (size_t)nn->d.V;
    if (rho) NN_TRY(cudaMemcpyAsync(rho, nn->rho, n3 * 4, cudaMemcpyDeviceToHost, nn->stream));
    if (mask) NN_TRY(cudaMemcpyAsync(mask, nn->mask, n3 * 4, cudaMemcpyDeviceToHost, nn->stream));
    NN_TRY(cudaStreamSynchronize(nn->stream));
    return SVL_OK;
}

}  // namespace svl
