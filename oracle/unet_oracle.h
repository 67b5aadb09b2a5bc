/* CPU oracle of the learned preconditioner network (TEST INFRASTRUCTURE ONLY). */
#ifndef UNET_ORACLE_H
#define UNET_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define UO_NLAYERS 15
#define UO_NTENSORS 16

typedef struct {
    int cin, cout, stride, relu, level;
    int in, in_cs, in_c0;
    int out, out_cs, out_c0;
    int woff, boff;
} uo_layer;

/* fills the 15-layer table, returns the parameter count */
int uo_layers(int c0, uo_layer *L);
int uo_nparams(int c0);

/* H and W must be 8k+1 so that the four levels nest.
 * loss (masked mean squared error), the network output [B][H][W][2] and the
 * parameter gradient (if grad != NULL); input [B][H][W][8], target and mask
 * [B][H][W][2] (mask may be NULL) */
double uo_loss_grad(const float *params, int c0, int B, int H, int W, const float *input, const float *target,
                    const float *mask, int bf16, float *out, float *grad);

#ifdef __cplusplus
}
#endif
#endif
