/*
 * pdal_learn.h -- the learned warm start of libpdal_learn_gb300.so: a
 * three-layer MLP (ReLU hidden layers, linear output) trained and evaluated
 * on the GPU by the library's own CUDA kernels.
 *
 * It maps instance features (costs, supplies, demands, capacities of a
 * transportation LP) to a predicted primal/dual warm start and an initial
 * sigma; the LP solver still runs to its own KKT tolerance.  None of these
 * functions has a counterpart in the reference, which has no learned
 * component.
 *
 * Parameters are FP32, stored layer by layer as W1 (in x hidden, row-major),
 * b1, W2 (hidden x hidden), b2, W3 (hidden x out), b3.  Training minimises the
 * mean squared error over all outputs with Adam.  Functions returning int give
 * 0 on success and -1 on failure (message in pdal_mlp_last_error).
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pdal_mlp pdal_mlp_t;

/* Random initialisation (He-uniform weights, zero biases) from `seed`, on
 * `device` (-1: current). NULL on failure. */
pdal_mlp_t *pdal_mlp_create(int in, int hidden, int out, unsigned seed, int device);
void pdal_mlp_free(pdal_mlp_t *mlp);

long long pdal_mlp_num_params(const pdal_mlp_t *mlp);
int pdal_mlp_get_params(const pdal_mlp_t *mlp, float *params);
int pdal_mlp_set_params(pdal_mlp_t *mlp, const float *params);

/* Uploads a training set: X is n x in, Y is n x out (row-major FP32). */
int pdal_mlp_set_data(pdal_mlp_t *mlp, int n, const float *X, const float *Y);

/* Adam epochs over the uploaded set in shuffled minibatches (the shuffle
 * from `seed`); returns the mean loss of the last epoch, or a negative value
 * on failure. */
double pdal_mlp_train(pdal_mlp_t *mlp, int epochs, int batch, float lr, unsigned seed);

/* Mean squared error of (X, Y) and, if grad != NULL, its gradient with
 * respect to every parameter (same layout as the parameters); one forward
 * and backward pass over all n rows.  Negative on failure. */
double pdal_mlp_loss_grad(pdal_mlp_t *mlp, int n, const float *X, const float *Y, float *grad);

/* Forward pass of n rows. bf16 != 0: weights and activations rounded to
 * BF16, products accumulated in FP32; bf16 == 0: FP32 throughout. */
int pdal_mlp_predict(pdal_mlp_t *mlp, int n, const float *X, float *Y, int bf16);

/* The transportation family on the device.  `count` instances of an S x D
 * complete bipartite transportation LP (arc a = i*D + j, supply rows i, demand
 * rows S + j, 0 <= x_a <= cap_a): costs and caps are count x (S*D), rhs is
 * count x (S+D) (supplies, then demands), row-major host arrays.  For each
 * instance the GPU forms the MLP's input (costs / 100, caps / 200, rhs / 100,
 * standardised with xm, xs: in = 2 S D + S + D entries), runs the network
 * (bf16 as in pdal_mlp_predict), decodes its output t = T * ys + ym
 * (out = S D + S + D + 1 entries) into x = clip(t[:SD], 0, 1) * cap,
 * y = 100 t[SD : SD+S+D], sigma = exp(t[last]), and evaluates the relative KKT
 * error max(|A x - b| / (1 + |b|), |c'x - d(y)| / (1 + |c'x| + |d(y)|)),
 * d(y) = b'y + sum min(c - A'y, 0) cap, of that point (kkt_pred) and of the
 * cold start x = 0, y = 0 (kkt_cold).  Outputs are host arrays of count x
 * (S*D), count x (S+D) and count entries. */
int pdal_transport_warm_start(pdal_mlp_t *mlp, int S, int D, int count, const double *costs, const double *caps,
                              const double *rhs, const double *xm, const double *xs, const double *ym,
                              const double *ys, int bf16, double *x, double *y, double *sigma, double *kkt_pred,
                              double *kkt_cold);

const char *pdal_mlp_last_error(void);

#ifdef __cplusplus
} /* extern "C" */
#endif
