/* mlp_oracle.c -- FP64 CPU restatement of the library's admissibility network.
 *
 * TEST INFRASTRUCTURE ONLY: the GPU's forward and backward kernels are
 * checked against these loops.  The reference has no learned component; the
 * network is defined here by its mathematics: layers 8 -> w -> w -> w -> 1
 * (hidden width w = 64 or 128), y = W x + b, ReLU after every layer but the last, loss = mean over
 * the batch of (y_hat - y)^2.  Parameter layout: per layer the weights
 * (out x in, row-major) then the biases.
 */
#include <stdlib.h>
#include <string.h>

#define NL 4
static int dims[NL + 1] = {8, 64, 64, 64, 1};

/* The hidden width (64 or 128, as the library's network). */
void orc_mlp_set_width(int w)
{
    if (w == 64 || w == 128) dims[1] = dims[2] = dims[3] = w;
}

int orc_mlp_param_count(void)
{
    int n = 0;
    for (int l = 0; l < NL; l++) n += dims[l + 1] * dims[l] + dims[l + 1];
    return n;
}

/* forward of one sample; acts[l] holds layer l's output (post-ReLU), acts[0] = x */
static void forward(const float *p, const float *x, double acts[NL + 1][128])
{
    for (int k = 0; k < dims[0]; k++) acts[0][k] = x[k];
    const float *q = p;
    for (int l = 0; l < NL; l++) {
        const int in = dims[l], out = dims[l + 1];
        const float *W = q, *b = q + (size_t)out * in;
        for (int o = 0; o < out; o++) {
            double s = b[o];
            for (int i = 0; i < in; i++) s += (double)W[(size_t)o * in + i] * acts[l][i];
            acts[l + 1][o] = (l + 1 < NL && s < 0.0) ? 0.0 : s;
        }
        q += (size_t)out * in + out;
    }
}

/* Predictions of n samples. */
void orc_mlp_forward(const float *p, const float *X, int n, double *out)
{
    double acts[NL + 1][128];
    for (int s = 0; s < n; s++) {
        forward(p, X + (size_t)s * dims[0], acts);
        out[s] = acts[NL][0];
    }
}

/* Mean squared error of a batch and its gradient (FP64). */
void orc_mlp_grad(const float *p, const float *X, const float *y, int n, double *grad, double *loss)
{
    const int np = orc_mlp_param_count();
    memset(grad, 0, (size_t)np * sizeof(double));
    double acts[NL + 1][128], delta[NL + 1][128];
    double L = 0.0;
    for (int s = 0; s < n; s++) {
        forward(p, X + (size_t)s * dims[0], acts);
        const double d = acts[NL][0] - (double)y[s];
        L += d * d;
        delta[NL][0] = 2.0 * d / (double)n;
        /* walk the layers backwards; offsets of each layer's parameters */
        size_t off[NL];
        size_t o0 = 0;
        for (int l = 0; l < NL; l++) {
            off[l] = o0;
            o0 += (size_t)dims[l + 1] * dims[l] + dims[l + 1];
        }
        for (int l = NL - 1; l >= 0; l--) {
            const int in = dims[l], out = dims[l + 1];
            const float *W = p + off[l];
            double *gW = grad + off[l], *gb = grad + off[l] + (size_t)out * in;
            for (int o = 0; o < out; o++) {
                gb[o] += delta[l + 1][o];
                for (int i = 0; i < in; i++) gW[(size_t)o * in + i] += delta[l + 1][o] * acts[l][i];
            }
            if (l > 0)
                for (int i = 0; i < in; i++) {
                    double t = 0.0;
                    for (int o = 0; o < out; o++) t += delta[l + 1][o] * (double)W[(size_t)o * in + i];
                    delta[l][i] = acts[l][i] > 0.0 ? t : 0.0;
                }
        }
    }
    *loss = L / (double)n;
}
