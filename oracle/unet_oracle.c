/* CPU oracle of the learned preconditioner network (TEST INFRASTRUCTURE ONLY).
 *
 * Loaded by tests/ (gradient checks of the GPU forward/backward kernels) and
 * nothing else.  The reference has no learned part: this is the restatement of
 * the network that pansfem2_gb300/csrc/psf_unet.cu implements, written as
 * plain loops in double precision so that it can be checked against finite
 * differences.  With bf16 = 1 it rounds the quantities the GPU stores in
 * bfloat16 (weights, activations, upsampled activations, pre-activation
 * gradients) to bfloat16 at the same points, round-to-nearest-even.
 *
 * Network: 4-level U-Net on a vertex-centred node grid (H, W odd so that the
 * stride-2 levels nest: H_l = (H_{l-1} + 1) / 2), channels c0, 2c0, 4c0, 8c0,
 * 3x3 convolutions, ReLU, stride-2 3x3 convolutions down, bilinear vertex
 * prolongation up, skip connections by channel concatenation, a final 3x3
 * convolution to 2 channels.  Inputs have 8 channels (density, 2 residual
 * components, the four surrounding element moduli, 1 zero).  Parameter layout per layer: W[co][tap][ci] then
 * b[co], tap = 3*dy + dx for offsets (dy-1, dx-1).  Loss: masked mean squared
 * error of the 2-channel output.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "unet_oracle.h"

static float rb16(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    memcpy(&x, &u, 4);
    return x;
}

static double R(double x, int bf16) { return bf16 ? (double)rb16((float)x) : x; }

int uo_layers(int c0, uo_layer *L) {
    /* in/out tensors: 0 input(8), 1 e0a, 2 cat0(c0|2c0), 3 e1a, 4 cat1(2c0|4c0), 5 e2a,
       6 cat2(4c0|8c0), 7 e3a, 8 e3, 9 d2a, 10 d2, 11 d1a, 12 d1, 13 d0a, 14 d0, 15 out */
    const int c1 = 2 * c0, c2 = 4 * c0, c3 = 8 * c0;
    uo_layer t[UO_NLAYERS] = {
        /* cin, cout, stride, relu, level, in, in_cs, in_c0, out, out_cs, out_c0 */
        {8, c0, 1, 1, 0, 0, 8, 0, 1, c0, 0},
        {c0, c0, 1, 1, 0, 1, c0, 0, 2, c0 + c1, 0},
        {c0, c1, 2, 1, 1, 2, c0 + c1, 0, 3, c1, 0},
        {c1, c1, 1, 1, 1, 3, c1, 0, 4, c1 + c2, 0},
        {c1, c2, 2, 1, 2, 4, c1 + c2, 0, 5, c2, 0},
        {c2, c2, 1, 1, 2, 5, c2, 0, 6, c2 + c3, 0},
        {c2, c3, 2, 1, 3, 6, c2 + c3, 0, 7, c3, 0},
        {c3, c3, 1, 1, 3, 7, c3, 0, 8, c3, 0},
        {c2 + c3, c2, 1, 1, 2, 6, c2 + c3, 0, 9, c2, 0},
        {c2, c2, 1, 1, 2, 9, c2, 0, 10, c2, 0},
        {c1 + c2, c1, 1, 1, 1, 4, c1 + c2, 0, 11, c1, 0},
        {c1, c1, 1, 1, 1, 11, c1, 0, 12, c1, 0},
        {c0 + c1, c0, 1, 1, 0, 2, c0 + c1, 0, 13, c0, 0},
        {c0, c0, 1, 1, 0, 13, c0, 0, 14, c0, 0},
        {c0, 2, 1, 0, 0, 14, c0, 0, 15, 2, 0},
    };
    int off = 0;
    for (int l = 0; l < UO_NLAYERS; l++) {
        L[l] = t[l];
        L[l].woff = off;
        off += L[l].cout * 9 * L[l].cin;
        L[l].boff = off;
        off += L[l].cout;
    }
    return off;
}

int uo_nparams(int c0) {
    uo_layer L[UO_NLAYERS];
    return uo_layers(c0, L);
}

typedef struct {
    int H[4], W[4];
    int C[UO_NTENSORS], lev[UO_NTENSORS];
    double *t[UO_NTENSORS];  /* activations [B][H][W][C] */
    double *g[UO_NTENSORS];  /* gradients */
} net_t;

static void shapes(int c0, int H, int W, net_t *n) {
    n->H[0] = H;
    n->W[0] = W;
    for (int l = 1; l < 4; l++) {
        n->H[l] = (n->H[l - 1] + 1) / 2;
        n->W[l] = (n->W[l - 1] + 1) / 2;
    }
    const int c1 = 2 * c0, c2 = 4 * c0, c3 = 8 * c0;
    int C[UO_NTENSORS] = {8, c0, c0 + c1, c1, c1 + c2, c2, c2 + c3, c3, c3, c2, c2, c1, c1, c0, c0, 2};
    int lev[UO_NTENSORS] = {0, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
    for (int i = 0; i < UO_NTENSORS; i++) {
        n->C[i] = C[i];
        n->lev[i] = lev[i];
    }
}

static size_t tsize(const net_t *n, int B, int i) {
    return (size_t)B * n->H[n->lev[i]] * n->W[n->lev[i]] * n->C[i];
}

/* input position of output (y, x) for tap (dy, dx); -1 when outside */
static int in_pos(int stride, int y, int x, int dy, int dx, int Hi, int Wi, int *yi, int *xi) {
    int a = stride * y + dy - 1, b = stride * x + dx - 1;
    if (a < 0 || a >= Hi || b < 0 || b >= Wi) return 0;
    *yi = a;
    *xi = b;
    return 1;
}

static void conv_fwd(const uo_layer *ly, const double *Wt, const double *bias, const net_t *n, int B, int bf16) {
    const double *X = n->t[ly->in];
    double *Y = n->t[ly->out];
    int li = n->lev[ly->in], lo = ly->level;
    int Hi = n->H[li], Wi = n->W[li], Ho = n->H[lo], Wo = n->W[lo];
    int ics = ly->in_cs, ocs = ly->out_cs;
    for (int b = 0; b < B; b++)
        for (int y = 0; y < Ho; y++)
            for (int x = 0; x < Wo; x++) {
                double *yo = Y + (((size_t)b * Ho + y) * Wo + x) * ocs + ly->out_c0;
                for (int co = 0; co < ly->cout; co++) {
                    double acc = 0.0;
                    for (int t = 0; t < 9; t++) {
                        int yi, xi;
                        if (!in_pos(ly->stride, y, x, t / 3, t % 3, Hi, Wi, &yi, &xi)) continue;
                        const double *xv = X + (((size_t)b * Hi + yi) * Wi + xi) * ics + ly->in_c0;
                        const double *w = Wt + ((size_t)co * 9 + t) * ly->cin;
                        for (int ci = 0; ci < ly->cin; ci++) acc += w[ci] * xv[ci];
                    }
                    acc += bias[co];
                    if (ly->relu && acc < 0.0) acc = 0.0;
                    yo[co] = (ly->out == UO_NTENSORS - 1) ? acc : R(acc, bf16);
                }
            }
}

/* bilinear vertex prolongation of tensor src (coarse) into channels [c0, c0+C) of dst (fine) */
static void upsample(const double *src, int C, int Hc, int Wc, double *dst, int dcs, int dc0, int Hf, int Wf, int B,
                     int bf16) {
    for (int b = 0; b < B; b++)
        for (int y = 0; y < Hf; y++)
            for (int x = 0; x < Wf; x++) {
                int y0 = y / 2, y1 = (y + 1) / 2, x0 = x / 2, x1 = (x + 1) / 2;
                double *d = dst + (((size_t)b * Hf + y) * Wf + x) * dcs + dc0;
                const double *s00 = src + (((size_t)b * Hc + y0) * Wc + x0) * C;
                const double *s01 = src + (((size_t)b * Hc + y0) * Wc + x1) * C;
                const double *s10 = src + (((size_t)b * Hc + y1) * Wc + x0) * C;
                const double *s11 = src + (((size_t)b * Hc + y1) * Wc + x1) * C;
                for (int c = 0; c < C; c++) d[c] = R(0.25 * (s00[c] + s01[c] + s10[c] + s11[c]), bf16);
            }
}

/* adjoint of upsample: coarse gradient += restriction of fine channels [c0, c0+C) */
static void restrict_add(const double *fine, int fcs, int fc0, int Hf, int Wf, double *coarse, int C, int Hc, int Wc,
                         int B) {
    for (int b = 0; b < B; b++)
        for (int y = 0; y < Hf; y++)
            for (int x = 0; x < Wf; x++) {
                int y0 = y / 2, y1 = (y + 1) / 2, x0 = x / 2, x1 = (x + 1) / 2;
                const double *f = fine + (((size_t)b * Hf + y) * Wf + x) * fcs + fc0;
                double *c00 = coarse + (((size_t)b * Hc + y0) * Wc + x0) * C;
                double *c01 = coarse + (((size_t)b * Hc + y0) * Wc + x1) * C;
                double *c10 = coarse + (((size_t)b * Hc + y1) * Wc + x0) * C;
                double *c11 = coarse + (((size_t)b * Hc + y1) * Wc + x1) * C;
                for (int c = 0; c < C; c++) {
                    double v = 0.25 * f[c];
                    c00[c] += v;
                    c01[c] += v;
                    c10[c] += v;
                    c11[c] += v;
                }
            }
}

static void conv_bwd(const uo_layer *ly, const double *Wt, net_t *n, int B, int bf16, double *gW, double *gb,
                     int need_dx) {
    const double *X = n->t[ly->in];
    const double *Y = n->t[ly->out];
    double *GX = n->g[ly->in];
    const double *GY = n->g[ly->out];
    int li = n->lev[ly->in], lo = ly->level;
    int Hi = n->H[li], Wi = n->W[li], Ho = n->H[lo], Wo = n->W[lo];
    int ics = ly->in_cs, ocs = ly->out_cs;
    double *gp = (double *)malloc(sizeof(double) * ly->cout);
    for (int b = 0; b < B; b++)
        for (int y = 0; y < Ho; y++)
            for (int x = 0; x < Wo; x++) {
                size_t po = (((size_t)b * Ho + y) * Wo + x) * ocs + ly->out_c0;
                for (int co = 0; co < ly->cout; co++) {
                    double g = GY[po + co];
                    if (ly->relu && !(Y[po + co] > 0.0)) g = 0.0;
                    gp[co] = R(g, bf16);
                    gb[co] += gp[co];
                }
                for (int t = 0; t < 9; t++) {
                    int yi, xi;
                    if (!in_pos(ly->stride, y, x, t / 3, t % 3, Hi, Wi, &yi, &xi)) continue;
                    size_t pi = (((size_t)b * Hi + yi) * Wi + xi) * ics + ly->in_c0;
                    for (int co = 0; co < ly->cout; co++) {
                        if (gp[co] == 0.0) continue;
                        double *gw = gW + ((size_t)co * 9 + t) * ly->cin;
                        const double *w = Wt + ((size_t)co * 9 + t) * ly->cin;
                        for (int ci = 0; ci < ly->cin; ci++) {
                            gw[ci] += gp[co] * X[pi + ci];
                            if (need_dx) GX[pi + ci] += gp[co] * w[ci];
                        }
                    }
                }
            }
    free(gp);
}

double uo_loss_grad(const float *params, int c0, int B, int H, int W, const float *input, const float *target,
                    const float *mask, int bf16, float *out, float *grad) {
    uo_layer L[UO_NLAYERS];
    int np = uo_layers(c0, L);
    net_t n;
    memset(&n, 0, sizeof(n));
    shapes(c0, H, W, &n);
    double *P = (double *)malloc(sizeof(double) * np);
    for (int i = 0; i < np; i++) P[i] = (double)params[i];
    /* weights are stored in bf16 for the products; biases stay fp32 */
    for (int l = 0; l < UO_NLAYERS; l++)
        for (int i = L[l].woff; i < L[l].boff; i++) P[i] = R(P[i], bf16);
    for (int i = 0; i < UO_NTENSORS; i++) {
        n.t[i] = (double *)calloc(tsize(&n, B, i), sizeof(double));
        n.g[i] = (double *)calloc(tsize(&n, B, i), sizeof(double));
    }
    size_t nin = tsize(&n, B, 0);
    for (size_t i = 0; i < nin; i++) n.t[0][i] = R(input[i], bf16);
    /* forward in layer order; the upsample steps sit before layers 8, 10, 12 */
    for (int l = 0; l < UO_NLAYERS; l++) {
        if (l == 8) upsample(n.t[8], n.C[8], n.H[3], n.W[3], n.t[6], n.C[6], 4 * c0, n.H[2], n.W[2], B, bf16);
        if (l == 10) upsample(n.t[10], n.C[10], n.H[2], n.W[2], n.t[4], n.C[4], 2 * c0, n.H[1], n.W[1], B, bf16);
        if (l == 12) upsample(n.t[12], n.C[12], n.H[1], n.W[1], n.t[2], n.C[2], c0, n.H[0], n.W[0], B, bf16);
        conv_fwd(&L[l], P + L[l].woff, P + L[l].boff, &n, B, bf16);
    }
    size_t nout = tsize(&n, B, UO_NTENSORS - 1);
    double msum = 0.0, loss = 0.0;
    for (size_t i = 0; i < nout; i++) msum += mask ? mask[i] : 1.0;
    if (msum <= 0.0) msum = 1.0;
    for (size_t i = 0; i < nout; i++) {
        double m = mask ? mask[i] : 1.0, d = n.t[15][i] - target[i];
        loss += m * d * d;
        n.g[15][i] = 2.0 * m * d / msum;
        if (out) out[i] = (float)n.t[15][i];
    }
    loss /= msum;
    if (grad) {
        double *G = (double *)calloc(np, sizeof(double));
        for (int l = UO_NLAYERS - 1; l >= 0; l--) {
            conv_bwd(&L[l], P + L[l].woff, &n, B, bf16, G + L[l].woff, G + L[l].boff, l > 0);
            if (l == 12) restrict_add(n.g[2], n.C[2], c0, n.H[0], n.W[0], n.g[12], n.C[12], n.H[1], n.W[1], B);
            if (l == 10) restrict_add(n.g[4], n.C[4], 2 * c0, n.H[1], n.W[1], n.g[10], n.C[10], n.H[2], n.W[2], B);
            if (l == 8) restrict_add(n.g[6], n.C[6], 4 * c0, n.H[2], n.W[2], n.g[8], n.C[8], n.H[3], n.W[3], B);
        }
        for (int i = 0; i < np; i++) grad[i] = (float)G[i];
        free(G);
    }
    for (int i = 0; i < UO_NTENSORS; i++) {
        free(n.t[i]);
        free(n.g[i]);
    }
    free(P);
    return loss;
}
