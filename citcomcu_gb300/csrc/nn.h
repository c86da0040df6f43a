// Warm-start network of the Stokes solve (internal interface of nn.cu).
//
// A 3D convolutional encoder-decoder on the node grid of one multigrid level
// (nx x ny x nz nodes, node v = z + nz*(x + nx*y) as the solver numbers them;
// (n - 1) divisible by 4 along every axis).  Two inputs per node (T and
// log10 of the viscosity), four outputs (three velocity components and the
// pressure, in scaled units).  Nine 3x3x3 convolutions over three resolutions
// (channels 16 / 32 / 64), BF16 weights and activations, FP32 accumulation on
// the tensor cores (tcgen05.mma, accumulators in tensor memory), FP32 master
// weights trained with Adam.
#pragma once

#include <cuda_runtime.h>

#include "level.h"

struct NnNet;

#define NN_LAYERS 9
#define NN_IN 2    // input channels used (padded to 16 on the device)
#define NN_OUT 4   // output channels used (padded to 16 on the device)
#define NN_CH 16   // padded channel count of the network's input and output tensors

// 0 on success; `err` receives a message otherwise
int nn_create(int nx, int ny, int nz, unsigned seed, cudaStream_t st, NnNet **out, char *err, size_t errlen);
void nn_destroy(NnNet *n);
int nn_param_count(const NnNet *n);  // public layout: per layer W[cout][cin][27] then b[cout], FP32
int nn_voxels(const NnNet *n);
int nn_get_params(NnNet *n, float *host);
int nn_set_params(NnNet *n, const float *host);
int nn_get_grads(NnNet *n, float *host);

// x16: device, V x 16 BF16 (channels 0, 1 used); y32: device, V x 16 FP32 (0..3 used)
int nn_forward(NnNet *n, const void *x16, float *y32);
// gradient accumulators and the loss sum to zero
int nn_zero_grads(NnNet *n);
// adds the gradient of scale * sum over nodes and channels 0..3 of (y - t)^2
// (t: device, V x 4 FP32) to the accumulators and the loss to the loss sum
int nn_accumulate(NnNet *n, const void *x16, const float *t, float scale);
int nn_adam(NnNet *n, float lr, float beta1, float beta2, float eps);
// loss sum since the last nn_zero_grads (synchronises the stream)
int nn_loss(NnNet *n, double *loss);
// nonzero when a bounded wait of a tensor-core kernel timed out (synchronises)
int nn_device_error(NnNet *n);
const float *nn_last_output(const NnNet *n);  // y of the last forward (device)

// Solver-side data movement between the multigrid levels and the network grid
// (level Lc is the network's, Lf the finest, r = (Lf.nox - 1) / (Lc.nox - 1)).
// `work` is FP64 scratch of Lc.nno + Lc.noz + 2 words that carries the
// state's temperature-anomaly RMS `a` from the inputs to the targets and the
// guess of the same state.
// inputs: channel 0 the temperature anomaly (T restricted to the coarse nodes
// by full weighting, minus its horizontal mean) / a; channel 1 log10 of the
// mean Gauss-point viscosity of the coarse elements around the node
void launch_nn_inputs(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, int r, const double *T, const double *evi_c, void *x16,
                      double *work);
// targets (after the inputs of the same state): fine U at the coarse nodes
// / (su a); nodal mean of the fine element pressures around the node minus
// the mean pressure, / (sp a)
void launch_nn_targets(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, int r, const double *U, const double *P, double su,
                       double sp, double *work, float *t);
// guess (after the inputs and the forward pass): coarse velocity vector
// y su a (3 per node, FP64) and fine element pressures y sp a + mp
// (trilinear interpolation of the nodal pressure output at element centres)
void launch_nn_guess(cudaStream_t st, const Lvl &Lf, const Lvl &Lc, int r, const float *y32, double su, double sp, double mp,
                     const double *work, double *Uc, double *P);
