/*
 * oracle_mlp.c -- FP64 oracle of the learned radiance cache network.
 *
 * TEST INFRASTRUCTURE.  The reference has no learned component; this file
 * defines the network the CUDA kernels implement, in double precision:
 *
 *   input  x in R^9: position (normalised to [0,1]^3 by the scene box),
 *          surface normal, direction;
 *   encoding e in R^216: for input i and frequency k = 0..11,
 *          e[(12 i + k) 2 + 0] = sin(2^k pi x_i), e[(12 i + k) 2 + 1] = cos(2^k pi x_i);
 *   network: h1 = relu(W0 e), h2 = relu(W1 h1), h3 = relu(W2 h2),
 *            h4 = relu(W3 h3), y = W4 h4  (no biases; W0 64x216, W1..W3 64x64,
 *            W4 3x64, row-major [out][in]);
 *   loss: relative L2 of Mueller et al. 2021 (neural radiance caching),
 *         L = 1/(3n) sum (y - t)^2 / (sg(y)^2 + 0.01), sg = stop-gradient;
 *   optimiser: Adam (Kingma & Ba 2015) with bias correction.
 *
 * Parameters are one flat array in the order W0, W1, W2, W3, W4.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>

#define NI 9
#define NF 12
#define NE 216
#define NH 64
#define NO 3

#define OFF_W0 0
#define OFF_W1 (OFF_W0 + NH * NE)
#define OFF_W2 (OFF_W1 + NH * NH)
#define OFF_W3 (OFF_W2 + NH * NH)
#define OFF_W4 (OFF_W3 + NH * NH)
#define N_PARAMS (OFF_W4 + NO * NH)

int oracle_mlp_n_params(void) { return N_PARAMS; }

static void encode(const float* x, double* e)
{
    for (int i = 0; i < NI; i++)
        for (int k = 0; k < NF; k++)
        {
            const double a = M_PI * ldexp((double)x[i], k);
            e[(i * NF + k) * 2 + 0] = sin(a);
            e[(i * NF + k) * 2 + 1] = cos(a);
        }
}

void oracle_mlp_encode(const float* x, uint32_t n, double* out)
{
    for (uint32_t s = 0; s < n; s++) encode(&x[s * NI], &out[(size_t)s * NE]);
}

/* y = W h for W [nout][nin] row-major */
static void matvec(const double* W, const double* h, int nout, int nin, double* y)
{
    for (int o = 0; o < nout; o++)
    {
        double a = 0.0;
        for (int i = 0; i < nin; i++) a += W[o * nin + i] * h[i];
        y[o] = a;
    }
}

static void forward1(const double* W, const float* x, double acts[5][NE], double y[NO])
{
    encode(x, acts[0]);
    const double* Ws[4] = { W + OFF_W0, W + OFF_W1, W + OFF_W2, W + OFF_W3 };
    const int nin[4] = { NE, NH, NH, NH };
    for (int l = 0; l < 4; l++)
    {
        matvec(Ws[l], acts[l], NH, nin[l], acts[l + 1]);
        for (int o = 0; o < NH; o++) if (acts[l + 1][o] < 0.0) acts[l + 1][o] = 0.0;
    }
    matvec(W + OFF_W4, acts[4], NO, NH, y);
}

void oracle_mlp_forward(const double* W, const float* x, uint32_t n, double* out)
{
#pragma omp parallel for schedule(static)
    for (int64_t s = 0; s < (int64_t)n; s++)
    {
        double acts[5][NE];
        forward1(W, &x[s * NI], acts, &out[s * NO]);
    }
}

/* loss and its gradient over a batch (gradient averaged over the batch) */
double oracle_mlp_loss_grad(const double* W, const float* x, const float* target, uint32_t n, double* grad)
{
    memset(grad, 0, sizeof(double) * N_PARAMS);
    double loss = 0.0;
    for (uint32_t s = 0; s < n; s++)
    {
        double acts[5][NE], y[NO], dy[NO], d4[NH], d3[NH], d2[NH], d1[NH];
        forward1(W, &x[s * NI], acts, y);
        for (int c = 0; c < NO; c++)
        {
            const double den = y[c] * y[c] + 0.01;
            const double r = y[c] - (double)target[s * NO + c];
            loss += r * r / den;
            dy[c] = 2.0 * r / den / (3.0 * n);
        }
        /* W4 and the delta into h4 */
        for (int c = 0; c < NO; c++)
            for (int i = 0; i < NH; i++) grad[OFF_W4 + c * NH + i] += dy[c] * acts[4][i];
        for (int i = 0; i < NH; i++)
        {
            double a = 0.0;
            for (int c = 0; c < NO; c++) a += W[OFF_W4 + c * NH + i] * dy[c];
            d4[i] = acts[4][i] > 0.0 ? a : 0.0;
        }
        double* dcur = d4;
        double* dnext[3] = { d3, d2, d1 };
        const int offs[4] = { OFF_W0, OFF_W1, OFF_W2, OFF_W3 };
        for (int l = 3; l >= 1; l--)
        {
            /* layer l maps acts[l] (64) -> acts[l+1]; its output delta is dcur */
            for (int o = 0; o < NH; o++)
                for (int i = 0; i < NH; i++) grad[offs[l] + o * NH + i] += dcur[o] * acts[l][i];
            double* dn = dnext[3 - l];
            for (int i = 0; i < NH; i++)
            {
                double a = 0.0;
                for (int o = 0; o < NH; o++) a += W[offs[l] + o * NH + i] * dcur[o];
                dn[i] = acts[l][i] > 0.0 ? a : 0.0;
            }
            dcur = dn;
        }
        for (int o = 0; o < NH; o++)
            for (int i = 0; i < NE; i++) grad[OFF_W0 + o * NE + i] += dcur[o] * acts[0][i];
    }
    return loss / (3.0 * n);
}

/* Adam, step t >= 1 */
void oracle_mlp_adam(double* W, double* m, double* v, const double* g, uint32_t n_params, uint32_t t, double lr,
                     double b1, double b2, double eps)
{
    const double c1 = 1.0 - pow(b1, (double)t), c2 = 1.0 - pow(b2, (double)t);
    for (uint32_t i = 0; i < n_params; i++)
    {
        m[i] = b1 * m[i] + (1.0 - b1) * g[i];
        v[i] = b2 * v[i] + (1.0 - b2) * g[i] * g[i];
        W[i] -= lr * (m[i] / c1) / (sqrt(v[i] / c2) + eps);
    }
}
