/*
 * foilcfd_wallnet.h - C ABI of the learned friction-velocity seed for the
 * iMEM wall model.
 *
 * The reference solves Reichardt's law for u_tau at every wall cell with six
 * FP32 Newton iterations from a warm seed (src/sim/lbm_wallmodel.cu:47-73, solveUTau).
 * This extension supplies the initial guess from a small network instead:
 *
 *     x = ((log u_par, log y, log nu) - in_mean) / in_std
 *     h1 = tanh(W1 x + b1)            W1: 32x3
 *     h2 = tanh(W2 h1 + b2)           W2: 32x32
 *     log u_tau = log u_par + out_mean + out_std * (W3 . h2 + b3)
 *
 * Weights are stored and applied as BF16 with FP32 accumulation; the
 * normalisation constants stay FP32. Inference (the seed solves and the
 * solver's learned wall update) runs the 32x32 layer on the tensor cores,
 * one warp's 32 samples per contraction, each FP32 activation split into
 * three BF16 terms. The network output is the logarithm of
 * u_tau (the fixed log u_par term only centres the target). One FP32 Newton
 * correction follows; when the relative Reichardt residual |g| / u_par after
 * it exceeds 1e-6, the cell falls back to full FP64 Newton (relative step
 * below 1e-8), which is also the reference the seed's error is measured against.
 *
 * The network is trained on the GPU by this library's own forward/backward
 * and Adam kernels from (u_par, y, nu, u_tau) samples: harvested from a
 * running solver's wall cells (fcfd_wall_harvest) and synthetic ones, with
 * labels from the FP64 Newton solve (fcfd_utau_solve, FCFD_UTAU_NEWTON64).
 *
 * None of these entry points has a counterpart in the reference; each names
 * the reference code it extends. All sample arrays are DEVICE pointers of n
 * FP32 values; `stream` is a cudaStream_t or NULL. Functions returning int
 * give 0 or a cudaError_t value. Not thread-safe (one host thread per net).
 */
#ifndef FOILCFD_WALLNET_H
#define FOILCFD_WALLNET_H

#include <stddef.h>
#include <stdint.h>

#include "foilcfd_step.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Parameter vector (FP32 master copy) layout: W1[32][3], b1[32], W2[32][32],
 * b2[32], W3[32], b3[1]. */
#define FCFD_WALLNET_HIDDEN 32
#define FCFD_WALLNET_PARAMS 1217

/* u_tau solve methods. */
enum {
    FCFD_UTAU_REFERENCE = 0,   /* 6 FP32 Newton iterations (fast intrinsics),
                                  warm seed if given else the reference's
                                  fresh seed max(0.04 u, sqrt(nu u / y))   */
    FCFD_UTAU_NEWTON64 = 1,    /* FP64 Newton to a relative step <= 1e-8,
                                  same seed rule ("full Newton")           */
    FCFD_UTAU_LEARNED = 2,     /* network seed, at most one FP32 Newton
                                  correction, FP64 fallback above 1e-6     */
    FCFD_UTAU_NEWTON64_NET = 3 /* FP64 Newton to 1e-8 from the network seed
                                  (solve-only: measures what the seed saves) */
};

typedef struct fcfd_wallnet fcfd_wallnet;

typedef struct fcfd_wallnet_norm {
    float in_mean[3], in_std[3]; /* of log u_par, log y, log nu            */
    float out_mean, out_std;     /* of log u_tau - log u_par               */
} fcfd_wallnet_norm;

typedef struct fcfd_wallnet_train_opts {
    int epochs;          /* passes over the samples                         */
    int batch;           /* samples per Adam step (multiple of 128)        */
    float lr_max;        /* one-cycle peak learning rate                   */
    float warmup_frac;   /* fraction of steps rising from lr_max/25        */
    float beta1, beta2, eps; /* Adam                                        */
    unsigned long long seed; /* epoch shuffles                              */
} fcfd_wallnet_train_opts;

/* Solve-side statistics of one batch of u_tau solves or one wall update. */
typedef struct fcfd_utau_stats {
    int solved;          /* samples / active wall cells solved              */
    int fallbacks;       /* of them: FP64 fallbacks (learned method)        */
    long long newton_iterations; /* FP64 iterations summed (methods 1, 3)   */
} fcfd_utau_stats;

fcfd_wallnet* fcfd_wallnet_create(void);
void fcfd_wallnet_destroy(fcfd_wallnet* net);

/* Xavier-uniform weights, zero biases, unit normalisation (seeded). */
int fcfd_wallnet_init_params(fcfd_wallnet* net, unsigned long long seed);
/* Host FP32 parameter vector (FCFD_WALLNET_PARAMS) + normalisation in/out;
 * get also returns the BF16-rounded weights the kernels apply (nullable). */
int fcfd_wallnet_set_params(fcfd_wallnet* net, const float* params, const fcfd_wallnet_norm* norm);
int fcfd_wallnet_get_params(const fcfd_wallnet* net, float* params, float* params_bf16, fcfd_wallnet_norm* norm);

/* Normalisation from n training samples (device arrays; FP64 sums). */
int fcfd_wallnet_fit_norm(fcfd_wallnet* net, const float* u_par, const float* y, const float* nu,
                          const float* u_tau, int n, void* stream);

/* Mean squared error (normalised log space) and its gradient over all n
 * samples at the current BF16 weights: loss -> *loss, gradient -> grad
 * (host, FCFD_WALLNET_PARAMS floats). For gradient checks. */
int fcfd_wallnet_gradient(fcfd_wallnet* net, const float* u_par, const float* y, const float* nu,
                          const float* u_tau, int n, double* loss, float* grad, void* stream);

/* Adam training (FP32 master weights, BF16 forward/backward, one-cycle
 * learning rate). loss_per_epoch (host, epochs floats, nullable) receives the
 * mean loss of each epoch's last step. */
int fcfd_wallnet_train(fcfd_wallnet* net, const float* u_par, const float* y, const float* nu,
                       const float* u_tau, int n, const fcfd_wallnet_train_opts* opts, float* loss_per_epoch,
                       void* stream);

/* Network seed only: u_tau_seed[i] for each sample. */
int fcfd_wallnet_predict(const fcfd_wallnet* net, const float* u_par, const float* y, const float* nu,
                         float* u_tau_seed, int n, void* stream);

/* u_tau for each sample by one of the FCFD_UTAU_* methods (net may be NULL
 * for methods 0 and 1; warm_seed nullable, used by methods 0 and 1 where
 * positive). stats (host, nullable) synchronises the stream. */
int fcfd_utau_solve(int method, const fcfd_wallnet* net, const float* u_par, const float* y, const float* nu,
                    const float* warm_seed, float* u_tau, int n, fcfd_utau_stats* stats, void* stream);

/* ---- solver integration (extends src/sim/lbm_wallmodel.cu:31-196) ------- */

/* Select the u_tau solve of the solver's wall updates: FCFD_UTAU_REFERENCE
 * (default, the reference's), FCFD_UTAU_NEWTON64 or FCFD_UTAU_LEARNED (net
 * required; its BF16 weights are copied, the net may be destroyed after). */
int fcfd_set_wall_solver(fcfd_solver* s, int method, const fcfd_wallnet* net);

/* Sampled tangential speed u_par and sample distance y of every wall-list
 * entry of a level (0 coarse, 1 fine) at the current state, into device
 * arrays of capacity >= fcfd_wall_count(s, level); entries below the
 * update's cut-off speed get u_par = 0. *count = entries written. */
int fcfd_wall_harvest(fcfd_solver* s, int level, float* u_par, float* y, int capacity, int* count);

/* Run `reps` wall updates of a level back to back with the selected method,
 * bracketed by CUDA events on the solver's stream: mean ms per update, and
 * the last update's solve statistics. Mutates u_tau and the slip field like
 * any wall update. */
int fcfd_wall_update_timed(fcfd_solver* s, int level, int reps, float* ms_per_update, fcfd_utau_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* FOILCFD_WALLNET_H */
