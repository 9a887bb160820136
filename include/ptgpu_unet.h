/*
 * ptgpu_unet.h -- the learned psi initial guess (no reference counterpart: the reference starts
 * every multigrid solve from the previous psi, iterative_solver.f90:124-160).
 *
 * A 4-level U-Net, base width 32: 3x3 convolutions with ReLU (two per level), 2x2 average
 * pooling, nearest-neighbour upsampling with skip concatenation, a 1x1 linear output.  Inputs
 * are 4 channels on the H x W = nz x nx grid of nodes (i < nx, k < nz): T, C, log10(eta)/5 and
 * RHS / max|RHS|; the output is psi / max|psi|.  BF16 weights and activations, FP32
 * accumulation on the tcgen05 tensor cores (implicit-GEMM forward, backward-data and
 * backward-weight convolutions), FP32 master weights and Adam.  H and W must be multiples of 8.
 *
 * Parameter layout (FP32, flat): for each of the 14 convolutions in order (e1a e1 e2a e2 e3a e3 b1
 * b2 d3a d3 d2a d2 d1a d1) w[cout][9][cin] (tap = 3*(dy+1) + (dx+1)) then b[cout]; then the 1x1
 * output w[32] and b[1].  Channel counts: 4-32, 32-32, 32-64, 64-64, 64-128, 128-128, 128-256,
 * 256-256, (256+128)-128, 128-128, (128+64)-64, 64-64, (64+32)-32, 32-32.
 * Host arrays: x [B][4][H][W], target and output [B][H][W], all FP32.
 */
#ifndef PTGPU_UNET_H
#define PTGPU_UNET_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pt_unet pt_unet;

int pt_unet_create(int nz, int nx, int max_batch, uint64_t seed, pt_unet** out);
int pt_unet_destroy(pt_unet* net);
int pt_unet_num_params(pt_unet* net, int64_t* n);
int pt_unet_get_params(pt_unet* net, float* host);
int pt_unet_set_params(pt_unet* net, const float* host);
/* forward pass of a batch (batch <= max_batch) */
int pt_unet_forward(pt_unet* net, const float* x, int batch, float* y);
/* loss = mean (y - target)^2 and its gradient w.r.t. every parameter (flat layout above) */
int pt_unet_gradients(pt_unet* net, const float* x, const float* target, int batch, float* grads, float* loss);
/* one Adam step (beta 0.9/0.999, eps 1e-8) on a batch; loss before the step */
int pt_unet_train_step(pt_unet* net, const float* x, const float* target, int batch, float lr, float* loss);
/* weight file: "PTUNET01", int32 nz, int32 nx, int64 nparams, FP32 parameters */
int pt_unet_save(pt_unet* net, const char* path);
int pt_unet_load(const char* path, int nz, int nx, int max_batch, pt_unet** out);

/* Device time of each of the 14 convolution GEMMs of one forward pass (CUDA events on the network's
 * stream, after a warm-up pass): ms[l] for layer l (4 levels x width 32, see the weight layout). */
int pt_unet_profile_forward(pt_unet* net, const float* x, int batch, float* ms);

/* Training pair of the current engine state (after pt_solve_psi): the network's input planes
 * x4 [4][nz][nx] (T, C, log10(eta)/5, RHS/max|RHS|) and the target psi/max|psi| [nz][nx], on
 * nodes i < nx, k < nz.  The FP64 solver's own output, written out for training. */
int pt_training_pair(float* x4, float* psi);

/* Training pairs of a time-evolved run: after pt_pair_capture(capacity), every converged psi solve
 * (pt_solve_psi and the RK-stage solves inside pt_step) appends its pair (as pt_training_pair
 * writes it) to a device buffer of `capacity` pairs; solves beyond capacity are not recorded.
 * pt_pair_take copies up to max_pairs of them (x4: [n][4][nz][nx], psi: [n][nz][nx]), sets *taken,
 * and empties the buffer.  capacity 0 stops capturing and frees the buffer. */
int pt_pair_capture(int capacity);
int pt_pair_take(float* x4, float* psi, int max_pairs, int* taken);

/* Outcome of the last solve's learned guess (pt_set_guess_mode(PT_GUESS_UNET, path)).  The
 * network's psi shape is scaled by the least-squares factor fitted on the coarsest multigrid level;
 * the previous psi and the scaled guess each get the level-1 smoothing of a cycle and the one with
 * the lower residual starts the solve.  used = 1 when the network's guess won; resid_prev and
 * resid_net are the two mean|r| / mean|RHS| after that smoothing. */
int pt_unet_guess_info(int* used, double* resid_prev, double* resid_net);

/* Tensor-core GEMM self-check: C (M x N, FP32) = A (M x K) * B (N x K)^T with BF16 operands
 * (uint16 bit patterns); N a multiple of 16 in [16, 256]. */
int pt_tc_gemm_check(const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K);

#ifdef __cplusplus
}
#endif
#endif
