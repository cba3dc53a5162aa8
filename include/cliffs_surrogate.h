/* cliffs_surrogate.h -- a learned surrogate of the solver for source studies.
 *
 * No reference counterpart: the reference is the solver only.  The surrogate
 * is a multilayer perceptron, with an optional conv decoder for a map,
 * mapping a source's parameters to quantities of
 * interest of the run (gauge maxima, a max-inundation map), trained on
 * runs of the batched solver (cliffs_batch_*) and used with an ensemble of
 * independently initialised members whose disagreement sends a scenario back
 * to the solver.  Training and inference run on the GPU in hand-written
 * kernels: BF16 tensor-core matrix products with FP32 accumulation
 * (tcgen05.mma with accumulators in tensor memory and TMA-staged operands for
 * products of at least 128 rows, 16 columns and a 64-wide reduction;
 * mma.sync m16n8k16 for smaller ones), fused bias and ReLU, Adam in FP32
 * with BF16 copies of the weights.  Data are plain row-major FP32 host
 * arrays; the library keeps its own device copies.  Every call returns a
 * CLIFFS_* status (cliffs_gpu.h). */
#ifndef CLIFFS_SURROGATE_H
#define CLIFFS_SURROGATE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cliffs_mlp cliffs_mlp;

typedef struct cliffs_mlp_desc {
  int32_t n_in;   /* inputs (1..16) */
  int32_t width;  /* hidden width (multiple of 16, <= 4096) */
  int32_t depth;  /* hidden layers (1..16) */
  int32_t n_out;  /* dense outputs (1..16384) */
  uint64_t seed;  /* weight initialisation (He uniform) */
  /* Optional map decoder (map_side = 0: none).  The last dense layer then
   * also emits a latent grid of (map_side/8)^2 cells with map_ch[0]
   * channels; the decoder takes it through a ReLU and three levels, each a
   * 2x nearest-neighbour upsampling and a 3x3 convolution (zero padding)
   * with a bias: map_ch[0] -> map_ch[1] -> map_ch[2] channels with ReLUs,
   * then map_ch[2] -> 1 channel, a map_side x map_side map.  map_side: a
   * multiple of 8, <= 512; channels: multiples of 8, <= 64.  A level with 16
   * or more output channels runs as a BF16 tensor-core product (im2col,
   * FP32 accumulation), one with fewer as a direct convolution (FP32 sums of
   * BF16 products); weight and input gradients are direct FP32 sums of BF16
   * products in a fixed order.  Batches with a map are limited to
   * batch * map_side^2 * 16 < 2^31 (CLIFFS_ERR_ARG otherwise). */
  int32_t map_side;
  int32_t map_ch[3];
} cliffs_mlp_desc;

int cliffs_mlp_create(const cliffs_mlp_desc *d, cliffs_mlp **out);
void cliffs_mlp_destroy(cliffs_mlp *m);
/* Number of layers (depth + 1, plus 3 decoder levels with a map) and the
 * shape of layer l's weight (rows = outputs, cols = inputs; a decoder level:
 * rows = output channels, cols = 9 * input channels, the tap (ty*3 + tx)
 * major and the input channel minor). */
int cliffs_mlp_layers(const cliffs_mlp *m, int32_t *n_layers);
int cliffs_mlp_shape(const cliffs_mlp *m, int32_t layer, int32_t *rows, int32_t *cols);

/* Parameters and gradients of layer l: which = 0 weight (rows x cols), 1 bias
 * (rows), 2 weight gradient, 3 bias gradient (of the last
 * cliffs_mlp_gradients or training step). */
int cliffs_mlp_get(const cliffs_mlp *m, int32_t layer, int32_t which, float *host, int64_t n);
int cliffs_mlp_set(cliffs_mlp *m, int32_t layer, int32_t which, const float *host, int64_t n);

/* y (batch x n_y) = f(x (batch x n_in)); n_y = n_out, plus map_side^2 map
 * cells (row-major) after the dense outputs with a map decoder. */
int cliffs_mlp_predict(cliffs_mlp *m, int32_t batch, const float *x, float *y);
/* Loss and gradients of every parameter for one batch, without an update.
 * batch: multiple of 16.  Targets t: batch x n_y, laid out as y.  The loss
 * is the mean squared error over the batch and the dense outputs, plus that
 * over the batch and the map cells with a map decoder. */
int cliffs_mlp_gradients(cliffs_mlp *m, int32_t batch, const float *x, const float *t, float *loss);
/* Train with Adam on n samples (x: n x n_in, t: n x n_y): `epochs` passes
 * over a seeded shuffle in batches of `batch` (multiple of 16; the last
 * partial batch of an epoch is left out), learning rate lr with a cosine
 * decay to lr/20, decoupled weight decay weight_decay on the weights (not the
 * biases).  losses (epochs) gets each epoch's mean batch loss. */
int cliffs_mlp_train(cliffs_mlp *m, int32_t n, const float *x, const float *t, int32_t epochs, int32_t batch,
                     float lr, float weight_decay, uint64_t seed, float *losses);
/* Kernels launched so far. */
int cliffs_mlp_launch_count(const cliffs_mlp *m, int64_t *n);

#ifdef __cplusplus
}
#endif
#endif
