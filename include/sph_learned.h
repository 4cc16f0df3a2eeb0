/*
 * sph_learned.h -- learned relaxation for libsph_cuda.  No counterpart in
 * the reference: it replaces most of the work of double_density_relaxation
 * (fluid.c:541-611), which stays as the fallback and the reference for
 * training.
 *
 * Model.  A message-passing network over each particle's neighbours within h
 * (particles with more than 48 take the plain relaxation): messages are the
 * neighbour offsets, relative velocities, densities and near densities,
 * weighted by (1 - r/h)^p and aggregated into a 32-wide feature row, joined
 * with the particle's own density and near density and its scene's
 * stiffness ratios (the step's density pass computes every density first,
 * then a walk of its hit masks gathers the messages); a 2-layer
 * width-128 GELU MLP
 * maps the row to the relaxation displacement (in units of
 * s = h dt^2 (k + k_near + k_spring)) and to a predicted density error.
 * BF16 weights and activations, FP32 accumulation, on the tcgen05 tensor
 * cores (inference and training).
 *
 * Use.  Collect training samples from plain-method states of any handle
 * (sph_learned_collect), train (sph_learned_train), then attach the model
 * to a handle (sph_cuda_set_learned): its steps then use the network
 * wherever the predicted density error is at most `threshold` (in units of
 * the rest density) and the particle has at most 48 neighbours, and the
 * plain relaxation everywhere else.
 */
#ifndef SPH_LEARNED_H
#define SPH_LEARNED_H

#include "sph_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sph_learned sph_learned_t;

/* Network sizes. */
#define SPH_LEARNED_IN 32
#define SPH_LEARNED_HIDDEN 128
#define SPH_LEARNED_OUT 16
#define SPH_LEARNED_MAX_NEIGHBORS 48

/* Creates a model with seeded random weights and room for max_samples
 * training samples. */
int sph_learned_create(sph_learned_t **out, int max_samples, unsigned long long seed);
int sph_learned_destroy(sph_learned_t *l);

/* Appends training samples taken from the state handle h's next step
 * relaxes (gravity, viscosity and prediction applied, cells rebuilt; h's
 * particle state itself does not advance): features and the plain
 * relaxation displacement (its gather form) of a `fraction` of the
 * particles with at most 48 neighbours, chosen by a hash of (particle id,
 * model seed, call count), until max_samples are held.  *added receives the
 * number appended.  The density record that sph_cuda_download reports is
 * replaced by that of the predicted state. */
int sph_learned_collect(sph_learned_t *l, sph_cuda_t *h, float fraction, int *added);

/* Samples held, and dropping them all. */
int sph_learned_num_samples(sph_learned_t *l);
int sph_learned_clear_samples(sph_learned_t *l);

/* Stage 1: trains the displacement outputs on the collected samples
 * (mean squared error, Adam, FP32 master weights).  Stage 2 (calibrate):
 * on the handle's current state, measures the density error each particle
 * gets from the network's displacement instead of the plain one and trains
 * the error output on it.  losses receive the last epoch's mean loss. */
int sph_learned_train(sph_learned_t *l, int epochs, int batch, float lr, float *loss);
int sph_learned_calibrate(sph_learned_t *l, sph_cuda_t *h, int epochs, float lr, float *loss);

/* Number of parameters and their values (FP32 master copy), for saving and
 * restoring a trained model. */
int sph_learned_num_params(void);
int sph_learned_get_params(sph_learned_t *l, float *out);
int sph_learned_set_params(sph_learned_t *l, const float *in);

/* Network outputs for host feature rows (n x 32, FP32, converted to BF16):
 * out (n x 16, FP32).  For tests of the tensor-core kernels. */
int sph_learned_forward(sph_learned_t *l, const float *features, int n, float *out);

/* Feature rows of the state handle h's next step relaxes (n x 32 FP32, by
 * particle id) and each particle's neighbour count (-1 where the particle
 * always takes the plain relaxation: a coincident neighbour or an
 * overflowing bucket). */
int sph_learned_features(sph_cuda_t *h, float *features, int *counts);

/* C[M x N] = A[M x K] . B[N x K]^T on the tcgen05 tensor cores, from FP32
 * host matrices rounded to BF16 (row-major), FP32 result.  For tests. */
int sph_learned_gemm_check(const float *A, const float *B, float *C, int M, int N, int K);

/* Every wait of the tensor-core kernels on an mbarrier is bounded (one
 * second of the GPU's global timer): a wait that gives up ends its kernel
 * with an error status
 * instead of hanging the GPU.  This runs one such wait on an mbarrier that
 * nothing arrives at; *gave_up = 1 when the bound worked. */
int sph_learned_wait_selftest(int *gave_up);

/* Attaches (or, with l == NULL, detaches) a trained model to a handle;
 * threshold is the largest predicted density error, in units of the rest
 * density, at which a particle uses the network (e.g. 0.01); a negative
 * threshold sends every particle to the plain relaxation.  The model must
 * outlive the attachment (detach before sph_learned_destroy). */
int sph_cuda_set_learned(sph_cuda_t *h, sph_learned_t *l, float threshold);

/* Particle-steps that used the network and that fell back to the plain
 * relaxation, since the model was attached.  Returns SPH_ERR_CUDA if a
 * tensor-core wait of the attached network gave up during those steps
 * (their results are then not valid). */
int sph_cuda_learned_counts(sph_cuda_t *h, unsigned long long *learned,
                            unsigned long long *fallback);

#ifdef __cplusplus
}
#endif

#endif /* SPH_LEARNED_H */
