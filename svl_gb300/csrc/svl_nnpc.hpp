// Learned preconditioner for the implicit effective-stiffness solve on
// lattice (structured) hexahedral meshes: a 4-layer 3D convolutional network
// on the node lattice, trained on residual/error pairs of the effective
// stiffness by the library's own forward and backward kernels, and applied
// inside a flexible conjugate gradient.  No counterpart in the reference,
// whose LinearSystem implementations are direct (EigenSolver, MumpsSolver)
// or PETSc KSP with PETSc's own preconditioners (PetscSolver.cc:53-150).
//
// Network (all convolutions 3x3x3, zero padding, no bias):
//   features [6]  = [r_hat ; rho * r_hat]    (r_hat = D^-1/2 r, rho = (4/dt^2 m) / D)
//   a0 = relu(conv 6 -> 16), a1 = relu(conv 16 -> 16), a2 = relu(conv 16 -> 16),
//   y  = conv 16 -> 3
//   z  = D^-1/2 (r_hat + y)                  (Jacobi plus a learned correction)
// Grids are channel-major fp32 [C][nz][ny][nx] over the node lattice;
// restrained dofs are zero in every input and are masked out of every output.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace svl {

constexpr int kNnIn = 6, kNnHid = 16, kNnOut = 3, kNnTaps = 27;
constexpr int kNnWeights = kNnTaps * (kNnIn * kNnHid + kNnHid * kNnHid * 2 + kNnHid * kNnOut);

struct NnPrecond;

// gmap[f] = c * V + node (node = x + nx (y + ny z)) of free dof f.
int nn_create(int nx, int ny, int nz, const std::vector<int32_t>& gmap, const std::vector<double>& sdinv,
              const std::vector<double>& rho, cudaStream_t stream, NnPrecond** out);
void nn_destroy(NnPrecond* nn);
// z = D^-1/2 (r_hat + net(r_hat)) on free dofs (device vectors), async on the stream.
int nn_apply(NnPrecond* nn, const double* r, double* z);
// Adds one training pair given in the scaled space (r_hat, e_hat), both free-dof
// device vectors, multiplied by `scale` (1 / |e_hat| normalises the pair).
int nn_record_pair(NnPrecond* nn, const double* rhat, const double* ehat, double scale);
int nn_num_pairs(const NnPrecond* nn);
// Adam on the recorded pairs; *loss = mean relative squared error over the
// last tenth of the iterations.
int nn_train(NnPrecond* nn, int iters, int batch, float lr, uint64_t seed, float* loss);
// Iterations [it_begin, it_end) of an `iters`-long Adam run (learning-rate
// schedule over the whole run; moments reset when it_begin == 0).
int nn_train_segment(NnPrecond* nn, int it_begin, int it_end, int iters, int batch, float lr, uint64_t seed, float* loss);
// Training windows: each sample is a random crop x crop x crop window of a
// pair (loss masked 4 voxels inside window faces interior to the lattice);
// 0 = whole lattice.
int nn_set_crop(NnPrecond* nn, int crop);
int nn_set_weights(NnPrecond* nn, const float* w);
int nn_get_weights(NnPrecond* nn, float* w);
// Device forward + loss + backward of one sample given as host grids
// (x: [3][V] r_hat, t: [3][V] e_hat); accumulates nothing, returns the loss
// sum and the weight gradient (kNnWeights floats).  Test hook.
int nn_loss_grad_host(NnPrecond* nn, const float* x, const float* t, float* loss, float* grad);
// Host copies of the rho and free-dof mask grids ([3][V] each).  Test hook.
int nn_get_grids(NnPrecond* nn, float* rho, float* mask);
// Network output y ([3][V]) for a host r_hat grid x ([3][V]); path 0 = FP32 CUDA
// cores, 1 = BF16 tensor cores.  Test hook.
int nn_forward_host(NnPrecond* nn, const float* x, float* y, int path);
// Inference path used by nn_apply (0 = FP32 CUDA cores, 1 = tensor cores, the default).
void nn_set_path(NnPrecond* nn, int path);
// SVL_OK, or an error if a tensor-core launch reported a bounded wait that gave up.
int nn_status(NnPrecond* nn);

}  // namespace svl
