/*
 * CPU oracle of the per-DOF MLP of the learned warm start.
 *
 * TEST INFRASTRUCTURE ONLY (checker for tests/ and __graft_entry__.smoke()).
 * The MLP has no counterpart in the reference; this file restates the
 * network math of the library so that its tensor-core kernels can be checked:
 * 80 inputs -> 64 -> 64 -> 64 -> 2, tanh on the hidden layers, weights as
 * four row-major [out][80] matrices (64, 64, 64, 16 rows) with the bias in the
 * column of the constant-1 input (70 in layer 1, 64 in the others).
 *
 * exact == 0 emulates the library's number formats: weights, inputs, hidden
 * activations, output gradients and backpropagated dZ rounded to BF16
 * (round to nearest even), products summed in double (the library sums in
 * FP32).  exact != 0 is plain double arithmetic on the FP32 weights, used to
 * validate this backward pass against finite differences.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define IN 80
#define HID 64
#define OUTP 16
#define OUT 2
#define NW (3 * HID * IN + OUTP * IN)

static float bf16_bits_to_float(uint16_t b) {
    uint32_t u = (uint32_t)b << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

static float round_bf16(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x; /* inf / nan */
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

static double R(double x, int exact) { return exact ? x : (double)round_bf16((float)x); }
static double T(double z, int exact) { return exact ? tanh(z) : (double)tanhf((float)z); }

static const float* layer_w(const float* w, int l) { return w + l * HID * IN; }

/* forward of one sample; a[l][80] inputs of layer l (a[0] = x), z[l][..] pre-activations */
static void fwd(const float* w, const uint16_t* x, int exact, double a[4][IN], double z[4][HID]) {
    for (int k = 0; k < IN; ++k) a[0][k] = bf16_bits_to_float(x[k]);
    for (int l = 0; l < 4; ++l) {
        const int rows = l == 3 ? OUTP : HID;
        const float* W = layer_w(w, l);
        for (int o = 0; o < rows && (l < 3 || o < OUT); ++o) {
            double s = 0.;
            for (int k = 0; k < IN; ++k) s += R(W[o * IN + k], exact) * a[l][k];
            z[l][o] = s;
        }
        if (l < 3) {
            for (int o = 0; o < HID; ++o) a[l + 1][o] = R(T(z[l][o], exact), exact);
            a[l + 1][HID] = 1.;
            for (int k = HID + 1; k < IN; ++k) a[l + 1][k] = 0.;
        }
    }
}

void orc_mlp_forward(const float* w, const uint16_t* X, int64_t n, int exact, float* pred) {
    double a[4][IN], z[4][HID];
    for (int64_t s = 0; s < n; ++s) {
        fwd(w, X + s * IN, exact, a, z);
        pred[2 * s] = (float)z[3][0];
        pred[2 * s + 1] = (float)z[3][1];
    }
}

/* gradient of L = sum_s sum_k (out_k - y_k)^2 / (2n) with respect to w; returns L */
double orc_mlp_gradient(const float* w, const uint16_t* X, const float* Y, int64_t n, int exact, float* grad) {
    static double G[NW];
    memset(G, 0, sizeof(G));
    double a[4][IN], z[4][HID], dz[HID], dh[HID];
    double loss = 0.;
    const float gscale = 1.0f / (float)n;
    for (int64_t s = 0; s < n; ++s) {
        fwd(w, X + s * IN, exact, a, z);
        double g[OUTP] = {0};
        for (int k = 0; k < OUT; ++k) {
            const double e = z[3][k] - (double)Y[2 * s + k];
            loss += e * e;
            g[k] = exact ? e / (double)n : (double)round_bf16(gscale * (float)e);
        }
        /* layer 4 */
        for (int o = 0; o < OUT; ++o)
            for (int k = 0; k < IN; ++k) G[3 * HID * IN + o * IN + k] += g[o] * a[3][k];
        for (int k = 0; k < HID; ++k) {
            double v = 0.;
            for (int o = 0; o < OUTP; ++o) v += R(layer_w(w, 3)[o * IN + k], exact) * g[o];
            dh[k] = v;
        }
        for (int l = 2; l >= 0; --l) {
            for (int o = 0; o < HID; ++o) {
                const double h = T(z[l][o], exact);
                dz[o] = R(dh[o] * (1. - h * h), exact);
            }
            for (int o = 0; o < HID; ++o)
                for (int k = 0; k < IN; ++k) G[l * HID * IN + o * IN + k] += dz[o] * a[l][k];
            if (l == 0) break;
            for (int k = 0; k < HID; ++k) {
                double v = 0.;
                for (int o = 0; o < HID; ++o) v += R(layer_w(w, l)[o * IN + k], exact) * dz[o];
                dh[k] = v;
            }
        }
    }
    /* padding entries carry no gradient */
    for (int i = 0; i < NW; ++i) {
        const int l = i < 3 * HID * IN ? i / (HID * IN) : 3;
        const int o = (i - l * HID * IN) / IN, k = i % IN;
        const int real = (l == 0 ? k <= 70 : k <= HID) && (l < 3 || o < OUT);
        grad[i] = real ? (float)G[i] : 0.f;
    }
    return loss / (2.0 * (double)n);
}
