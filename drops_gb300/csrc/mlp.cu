// Per-DOF MLP of the learned Krylov warm start, on the fifth-generation
// tensor cores (tcgen05 BF16 MMA, FP32 accumulators in tensor memory).
//
// Network: 80 inputs (70 features, a constant 1 that carries the bias, zero
// padding) -> 64 -> 64 -> 64 -> 2, tanh on the hidden layers.  Every layer is
// stored as one row-major [out][80] FP32 matrix whose bias sits in the column
// of the constant input (70 for the first layer, 64 for the others); the
// output layer is padded to 16 rows, the smallest MMA width, rows 2..15 zero.
// Weights, inputs and hidden activations are BF16, sums FP32.
//
// One CTA of 128 threads processes tiles of 128 samples: thread t owns sample
// row t, which is also tensor-memory lane t of every accumulator.
//   forward   D_l = H_{l-1} W_l^T        (A: samples x 80, B: W_l, N = 64 or 16)
//   backward  dH_{l-1} = dZ_l W_l          (A: samples x out, B: W_l^T)
//             dW_l = dZ_l^T H_{l-1}        (A: out x samples, B: H_{l-1}^T, M = 128 padded, N = 80)
// so every operand is K-major and stored by the threads in the layout of
// umma.cuh.  Gradients of one tile are drained from tensor memory into a
// per-tile slot in global memory; k_mlp_adam sums the slots of a mini-batch in
// a fixed order and applies Adam.  Every wait on the tensor cores is bounded;
// a timeout sets the error word and the kernel frees its tensor memory and
// returns.
#include <cmath>
#include <random>

#include "tf_internal.cuh"
#include "umma.cuh"

namespace tf {

constexpr int kIn = 80;       // input width of every layer (padded)
constexpr int kHid = 64;
constexpr int kOutPad = 16;
constexpr int kOut = 2;
constexpr int kTile = 128;    // samples per tile = MMA M = tensor-memory lanes
constexpr int kBias0 = 70;    // input column of the constant 1, first layer
constexpr int kBiasH = 64;    // same for the hidden layers
constexpr int kW1 = 0, kW2 = kHid * kIn, kW3 = 2 * kHid * kIn, kW4 = 3 * kHid * kIn;
constexpr int kWTotal = 3 * kHid * kIn + kOutPad * kIn;  // 16640
constexpr int kGradSlot = 4 * kHid * kIn;                 // floats per tile: [layer][64][80]
constexpr uint32_t kWaitLimit = 1u << 22;

// tensor-memory columns
constexpr uint32_t kColD1 = 0, kColD2 = 64, kColD3 = 128, kColD4 = 192, kColDH = 208, kColDW = 272;

// shared-memory layout (bytes)
constexpr int kSzWf = kHid * kIn * 2;          // 10240, forward W1..W3 ([64 x 80])
constexpr int kSzW4f = kOutPad * kIn * 2;      // 2560
constexpr int kSzR = kTile * kIn * 2;          // 20480, samples x 80
constexpr int kSzT = kIn * kTile * 2;          // 20480, 80 x samples
constexpr int kSzDZt = kTile * kTile * 2;      // 32768, 128 x samples
constexpr int kSzW4b = kHid * kOutPad * 2;     // 2048, W4^T [64 x 16]
constexpr int kSzWb = kHid * kHid * 2;         // 8192, W^T [64 x 64]
constexpr int kOffW1 = 0, kOffW2 = kOffW1 + kSzWf, kOffW3 = kOffW2 + kSzWf, kOffW4 = kOffW3 + kSzWf;
constexpr int kOffR0 = kOffW4 + kSzW4f + 512;  // keep 1 KB alignment: 33280 -> 33792
constexpr int kOffR1 = kOffR0 + kSzR;
constexpr int kSmemInfer = kOffR1 + kSzR;      // 74752
constexpr int kOffXt = kSmemInfer, kOffH1t = kOffXt + kSzT, kOffH2t = kOffH1t + kSzT, kOffH3t = kOffH2t + kSzT;
constexpr int kOffDZt = kOffH3t + kSzT;
constexpr int kOffW4b = kOffDZt + kSzDZt, kOffW3b = kOffW4b + kSzW4b, kOffW2b = kOffW3b + kSzWb;
constexpr int kSmemTrain = kOffW2b + kSzWb;    // 74752 + 81920 + 32768 + 2048 + 16384 = 207872
static_assert(kSmemTrain <= 227 * 1024, "training tile does not fit shared memory");
static_assert(kOffR0 % 1024 == 0 && kOffXt % 1024 == 0 && kOffDZt % 1024 == 0, "tile alignment");

struct MlpArgs {
    const __nv_bfloat16* X;  // [n][80] inputs
    const float* Y;          // [n][2] targets (training)
    int64_t n;
    int tile0, ntiles;       // tiles tile0 + j * tstride, j < ntiles
    int tstride;
    const __nv_bfloat16* W;  // [kWTotal] BF16 weights
    float* pred;             // [n][2] outputs (inference)
    float* grad;             // [ntiles][kGradSlot] (training)
    float* loss;             // [ntiles] sum of squared errors (training)
    float gscale;            // d loss / d output = gscale * (out - y)
    int* err;
};

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

// 8 consecutive K elements of row r (a whole 16-byte core-matrix row)
__device__ __forceinline__ void st_row8(unsigned char* base, int R, int r, int k0, const float* v) {
    __align__(16) __nv_bfloat16 h[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) h[i] = __float2bfloat16_rn(v[i]);
    *reinterpret_cast<uint4*>(base + umma::tile_off(R, r, k0)) = *reinterpret_cast<const uint4*>(h);
}

template <bool kTrain>
__global__ void __launch_bounds__(kTile, 1) k_mlp(MlpArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ float red[4];
    const int t = threadIdx.x, warp = t >> 5;
    constexpr uint32_t kCols = kTrain ? 512 : 256;

    // ---- weights into shared memory ----
    for (int i = t; i < kWTotal; i += kTile) {
        const __nv_bfloat16 w = a.W[i];
        int layer, o, k;
        if (i < kW4) { layer = i / (kHid * kIn); o = (i % (kHid * kIn)) / kIn; k = i % kIn; }
        else { layer = 3; o = (i - kW4) / kIn; k = (i - kW4) % kIn; }
        const int offs[4] = {kOffW1, kOffW2, kOffW3, kOffW4};
        *reinterpret_cast<__nv_bfloat16*>(smem + offs[layer] + umma::tile_off(layer == 3 ? kOutPad : kHid, o, k)) = w;
        if (kTrain && layer >= 1 && k < kHid) {
            // W_l^T as [in rows x out K] for dH = dZ W_l
            if (layer == 3) *reinterpret_cast<__nv_bfloat16*>(smem + kOffW4b + umma::tile_off(kHid, k, o)) = w;
            else *reinterpret_cast<__nv_bfloat16*>(smem + (layer == 2 ? kOffW3b : kOffW2b) + umma::tile_off(kHid, k, o)) = w;
        }
    }
    if (kTrain) {  // transposed activation tiles and dZ^T: rows that are never written stay zero
        for (int i = t; i < (4 * kSzT + kSzDZt) / 16; i += kTile)
            reinterpret_cast<uint4*>(smem + kOffXt)[i] = make_uint4(0, 0, 0, 0);
    }
    if (t == 0) umma::mbar_init(&mbar, 1);
    if (warp == 0) umma::tmem_alloc(&tmem_base, kCols);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tm = tmem_base;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    const uint32_t sbase = umma::smem_u32(smem);
    uint32_t phase = 0;
    bool ok = true;

    // All threads: publish shared-memory writes and finished tensor-memory
    // reads; thread 0 issues the MMAs of `issue`; everyone waits for their
    // completion.  A wait that runs out is retried once (MMAs still in
    // flight), then the CTA agrees on the failure and stops.
    auto run = [&](auto issue) -> bool {
        umma::fence_smem_async();
        umma::fence_before_sync();
        __syncthreads();
        if (t == 0) {
            umma::fence_after_sync();
            issue();
            umma::commit(&mbar);
        }
        bool done = umma::mbar_wait(&mbar, phase, kWaitLimit);
        if (!done) done = umma::mbar_wait(&mbar, phase, kWaitLimit);
        phase ^= 1u;
        umma::fence_after_sync();
        if (__syncthreads_or(!done)) ok = false;
        return ok;
    };
    // D = A (R_A rows, K = 16 * ks) * B (R_B rows)^T
    auto gemm = [&](uint32_t dcol, int offA, int RA, int offB, int RB, int ks, int M, int N) {
        const uint32_t id = umma::idesc_bf16_f32(M, N);
        for (int s = 0; s < ks; ++s)
            umma::mma_bf16(tm + dcol, umma::tile_desc(sbase + offA, RA, s), umma::tile_desc(sbase + offB, RB, s), id,
                           s > 0 ? 1u : 0u);
    };

    float loss_acc = 0.f;
    for (int j = blockIdx.x; j < a.ntiles && ok; j += gridDim.x) {
        const int tile = a.tile0 + j * a.tstride;
        const int64_t row = (int64_t)tile * kTile + t;
        const bool valid = row < a.n;
        // ---- inputs ----
        {
            uint4 xv[kIn / 8];
#pragma unroll
            for (int g = 0; g < kIn / 8; ++g)
                xv[g] = valid ? reinterpret_cast<const uint4*>(a.X + row * kIn)[g] : make_uint4(0, 0, 0, 0);
#pragma unroll
            for (int g = 0; g < kIn / 8; ++g) *reinterpret_cast<uint4*>(smem + kOffR0 + umma::tile_off(kTile, t, 8 * g)) = xv[g];
            if (kTrain) {
                const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(xv);
                for (int f = 0; f < kIn; ++f)
                    *reinterpret_cast<__nv_bfloat16*>(smem + kOffXt + umma::tile_off(kIn, f, t)) = h[f];
            }
        }
        // ---- forward ----
        const int rA[3] = {kOffR0, kOffR1, kOffR0};
        const int wF[3] = {kOffW1, kOffW2, kOffW3};
        const uint32_t dC[3] = {kColD1, kColD2, kColD3};
        const int hT[3] = {kOffH1t, kOffH2t, kOffH3t};
        for (int l = 0; l < 3 && ok; ++l) {
            if (!run([&] { gemm(dC[l], rA[l], kTile, wF[l], kHid, kIn / 16, kTile, kHid); })) break;
            const int out = l == 1 ? kOffR0 : kOffR1;
            for (int c = 0; c < kHid / 16; ++c) {
                float v[16];
                umma::tmem_ld16(tm + lane_base + dC[l] + 16 * c, v);
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = tanhf(v[i]);
                st_row8(smem + out, kTile, t, 16 * c, v);
                st_row8(smem + out, kTile, t, 16 * c + 8, v + 8);
                if (kTrain)
                    for (int i = 0; i < 16; ++i) st_bf16(smem + hT[l], umma::tile_off(kIn, 16 * c + i, t), v[i]);
            }
            float tail[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            st_row8(smem + out, kTile, t, kBiasH, tail);
            tail[0] = 0.f;
            st_row8(smem + out, kTile, t, kBiasH + 8, tail);
            if (kTrain) st_bf16(smem + hT[l], umma::tile_off(kIn, kBiasH, t), 1.f);
        }
        if (!ok || !run([&] { gemm(kColD4, kOffR1, kTile, kOffW4, kOutPad, kIn / 16, kTile, kOutPad); })) break;
        float o[16];
        umma::tmem_ld16(tm + lane_base + kColD4, o);
        if (!kTrain) {
            if (valid) {
                a.pred[2 * row] = o[0];
                a.pred[2 * row + 1] = o[1];
            }
            continue;
        }
        // ---- loss gradient ----
        float g[16] = {};
        if (valid) {
            const float e0 = o[0] - a.Y[2 * row], e1 = o[1] - a.Y[2 * row + 1];
            loss_acc += e0 * e0 + e1 * e1;
            g[0] = a.gscale * e0;
            g[1] = a.gscale * e1;
        }
        st_row8(smem + kOffR0, kTile, t, 0, g);
        st_row8(smem + kOffR0, kTile, t, 8, g + 8);
        st_bf16(smem + kOffDZt, umma::tile_off(kTile, 0, t), g[0]);
        st_bf16(smem + kOffDZt, umma::tile_off(kTile, 1, t), g[1]);
        float* gslot = a.grad + (size_t)j * kGradSlot;
        // layer 4 (index 3), then 3, 2, 1
        const int hPrevT[4] = {kOffXt, kOffH1t, kOffH2t, kOffH3t};
        const int wB[4] = {0, kOffW2b, kOffW3b, kOffW4b};
        for (int l = 3; l >= 0; --l) {
            const int kout = l == 3 ? kOutPad : kHid;  // K of dH = dZ W_l
            const int nout = l == 3 ? kOut : kHid;     // real rows of dW_l
            if (!run([&] {
                    if (l > 0) gemm(kColDH, kOffR0, kTile, wB[l], kHid, kout / 16, kTile, kHid);
                    gemm(kColDW, kOffDZt, kTile, hPrevT[l], kIn, kTile / 16, kTile, kIn);
                }))
                break;
            // drain dW_l rows [0, nout)
            if (warp * 32 < nout) {
                for (int c = 0; c < kIn / 16; ++c) {
                    float v[16];
                    umma::tmem_ld16(tm + lane_base + kColDW + 16 * c, v);
                    if (t < nout) {
                        float4* dst = reinterpret_cast<float4*>(gslot + (size_t)l * kHid * kIn + (size_t)t * kIn + 16 * c);
#pragma unroll
                        for (int q = 0; q < 4; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    }
                }
            }
            if (l == 0) break;
            // dZ_{l-1} = dH_{l-1} * (1 - tanh^2(D_{l-1}))
            for (int c = 0; c < kHid / 16; ++c) {
                float dh[16], d[16];
                umma::tmem_ld16(tm + lane_base + kColDH + 16 * c, dh);
                umma::tmem_ld16(tm + lane_base + dC[l - 1] + 16 * c, d);
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const float h = tanhf(d[i]);
                    dh[i] = valid ? dh[i] * (1.f - h * h) : 0.f;
                }
                st_row8(smem + kOffR0, kTile, t, 16 * c, dh);
                st_row8(smem + kOffR0, kTile, t, 16 * c + 8, dh + 8);
                for (int i = 0; i < 16; ++i) st_bf16(smem + kOffDZt, umma::tile_off(kTile, 16 * c + i, t), dh[i]);
            }
        }
        if (!ok) break;
        // per-tile loss
        float s = loss_acc;
        loss_acc = 0.f;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if ((t & 31) == 0) red[warp] = s;
        __syncthreads();
        if (t == 0) a.loss[j] = (red[0] + red[1]) + (red[2] + red[3]);
    }
    if (!ok && t == 0) atomicExch(a.err, 1);
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after_sync();
        umma::tmem_dealloc(tm, kCols);
    }
}

// Sum of the tile gradients of a mini-batch (fixed order) and one Adam step on
// the FP32 master weights; padding entries stay zero.  lr == 0 only writes the
// summed gradient (gradient checks).
__global__ void k_mlp_adam(int ntiles, const float* __restrict__ grad, float* __restrict__ w, float* __restrict__ m1,
                           float* __restrict__ m2, __nv_bfloat16* __restrict__ w16, float* __restrict__ gsum, float lr,
                           float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kWTotal) return;
    int layer, o, k;
    if (i < kW4) { layer = i / (kHid * kIn); o = (i % (kHid * kIn)) / kIn; k = i % kIn; }
    else { layer = 3; o = (i - kW4) / kIn; k = (i - kW4) % kIn; }
    const bool real = (layer == 0 ? k <= kBias0 : k <= kBiasH) && (layer < 3 || o < kOut);
    float g = 0.f;
    if (real)
        for (int s = 0; s < ntiles; ++s) g += grad[(size_t)s * kGradSlot + (size_t)layer * kHid * kIn + (size_t)o * kIn + k];
    if (gsum) gsum[i] = g;
    if (!real || lr == 0.f) return;
    const float a1 = b1 * m1[i] + (1.f - b1) * g;
    const float a2 = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a1;
    m2[i] = a2;
    const float wn = w[i] - lr * (a1 * c1) / (sqrtf(a2 * c2) + eps);
    w[i] = wn;
    w16[i] = __float2bfloat16_rn(wn);
}

__global__ void k_mlp_to_bf16(const float* __restrict__ w, __nv_bfloat16* __restrict__ w16) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kWTotal) w16[i] = __float2bfloat16_rn(w[i]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int mlp_ready(Context* c) {
    if (c->mlp_w.p) return TF_OK;
    return mlp_init(c, 1234);
}

int mlp_init(Context* c, uint64_t seed) {
    std::vector<float> w(kWTotal, 0.f);
    std::mt19937_64 gen(seed);
    // uniform(-s, s) with s = sqrt(6 / (fan_in + fan_out)) on the real entries, biases zero
    auto fill = [&](int off, int rows, int fan_in, int fan_out) {
        const double s = std::sqrt(6.0 / (fan_in + fan_out));
        std::uniform_real_distribution<double> U(-s, s);
        for (int o = 0; o < rows; ++o)
            for (int k = 0; k < fan_in; ++k) w[off + o * kIn + k] = (float)U(gen);
    };
    fill(kW1, kHid, kBias0, kHid);
    fill(kW2, kHid, kHid, kHid);
    fill(kW3, kHid, kHid, kHid);
    fill(kW4, kOut, kHid, kOut);
    return mlp_set_weights(c, w.data());
}

int mlp_set_weights(Context* c, const float* w) {
    TF_TRY(ensure(c, c->mlp_w, kWTotal));
    TF_TRY(ensure(c, c->mlp_m1, kWTotal));
    TF_TRY(ensure(c, c->mlp_m2, kWTotal));
    TF_TRY(ensure(c, c->mlp_w16, kWTotal));
    TF_CUDA(c, cudaMemcpyAsync(c->mlp_w.p, w, sizeof(float) * kWTotal, cudaMemcpyHostToDevice, c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->mlp_m1.p, 0, sizeof(float) * kWTotal, c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->mlp_m2.p, 0, sizeof(float) * kWTotal, c->stream));
    k_mlp_to_bf16<<<(kWTotal + 255) / 256, 256, 0, c->stream>>>(c->mlp_w.p, c->mlp_w16.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->mlp_step = 0;
    return TF_OK;
}

int mlp_get_weights(Context* c, float* w) {
    TF_TRY(mlp_ready(c));
    TF_CUDA(c, cudaMemcpyAsync(w, c->mlp_w.p, sizeof(float) * kWTotal, cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    return TF_OK;
}

static int mlp_err_reset(Context* c) {
    TF_CUDA(c, cudaMemsetAsync(c->status.p + 2, 0, sizeof(int), c->stream));
    return TF_OK;
}

static int mlp_err_check(Context* c) {
    int e = 0;
    TF_CUDA(c, cudaMemcpyAsync(&e, c->status.p + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (e) return set_err(c, TF_ERR_WATCHDOG, "mlp: a tensor-core wait timed out");
    return TF_OK;
}

static bool g_mlp_attr[2] = {false, false};

// Inference asks for 80 KB of shared memory although it uses 73 KB, so that at
// most two CTAs share an SM and their tensor-memory allocations (256 columns
// each) always fit the SM's 512 columns; training holds 512 columns and one
// CTA per SM (its 203 KB of shared memory allow no second).
constexpr int kSmemInferLaunch = 80 * 1024;
static_assert(kSmemInferLaunch >= kSmemInfer && 3 * (kSmemInferLaunch + 1024) > 227 * 1024, "inference occupancy");

template <bool kTrain>
static int mlp_launch(Context* c, const MlpArgs& a, int grid) {
    const int smem = kTrain ? kSmemTrain : kSmemInferLaunch;
    if (!g_mlp_attr[kTrain]) {
        TF_CUDA(c, cudaFuncSetAttribute(k_mlp<kTrain>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        g_mlp_attr[kTrain] = true;
    }
    k_mlp<kTrain><<<grid, kTile, smem, c->stream>>>(a);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

// pred[n][2] = MLP(X[n][80]), device pointers
int mlp_forward_dev(Context* c, const __nv_bfloat16* X, int64_t n, float* pred) {
    TF_TRY(mlp_ready(c));
    if (n <= 0) return TF_OK;
    MlpArgs a{};
    a.X = X;
    a.n = n;
    a.tile0 = 0;
    a.ntiles = (int)((n + kTile - 1) / kTile);
    a.tstride = 1;
    a.W = c->mlp_w16.p;
    a.pred = pred;
    a.err = c->status.p + 2;
    TF_TRY(mlp_err_reset(c));
    TF_TRY(mlp_launch<false>(c, a, std::min(a.ntiles, 2 * c->num_sms)));
    return mlp_err_check(c);
}

// One pass over n samples in mini-batches of mb_tiles tiles (strided tiles, so
// each mini-batch spans the whole sample range); lr == 0: the gradient of the
// whole set is accumulated into gsum instead (one mini-batch holding every
// tile) and the weights stay unchanged.
int mlp_epoch_dev(Context* c, const __nv_bfloat16* X, const float* Y, int64_t n, int mb_tiles, float lr, float* gsum,
                  double* loss) {
    TF_TRY(mlp_ready(c));
    const int ntiles = (int)((n + kTile - 1) / kTile);
    if (ntiles < 1) return set_err(c, TF_ERR_BAD_INPUT, "mlp: no samples");
    if (lr == 0.f || mb_tiles > ntiles || mb_tiles < 1) mb_tiles = ntiles;
    const int nb = (ntiles + mb_tiles - 1) / mb_tiles;  // mini-batches
    TF_TRY(ensure(c, c->mlp_grad, (size_t)mb_tiles * kGradSlot));
    TF_TRY(ensure(c, c->mlp_lossacc, (size_t)nb * mb_tiles));
    TF_TRY(mlp_err_reset(c));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int b = 0; b < nb; ++b) {
        const int cnt = (ntiles - b + nb - 1) / nb;  // tiles b, b + nb, ... < ntiles
        MlpArgs a{};
        a.X = X;
        a.Y = Y;
        a.n = n;
        a.tile0 = b;
        a.tstride = nb;
        a.ntiles = cnt;
        a.W = c->mlp_w16.p;
        a.grad = c->mlp_grad.p;
        a.loss = c->mlp_lossacc.p + (size_t)b * mb_tiles;
        // mean over the samples of this mini-batch and the two outputs
        int64_t samples = 0;
        for (int jj = 0; jj < cnt; ++jj) {
            const int64_t r0 = (int64_t)(b + jj * nb) * kTile;
            samples += std::min<int64_t>(kTile, n - r0);
        }
        a.gscale = 2.f / (2.f * (float)samples);
        a.err = c->status.p + 2;
        TF_TRY(mlp_launch<true>(c, a, std::min(cnt, c->num_sms)));
        double c1 = 1.0, c2 = 1.0;
        if (lr != 0.f) {
            ++c->mlp_step;
            c1 = 1.0 / (1.0 - std::pow(0.9, c->mlp_step));
            c2 = 1.0 / (1.0 - std::pow(0.999, c->mlp_step));
        }
        k_mlp_adam<<<(kWTotal + 255) / 256, 256, 0, c->stream>>>(cnt, c->mlp_grad.p, c->mlp_w.p, c->mlp_m1.p, c->mlp_m2.p,
                                                                 c->mlp_w16.p, gsum, lr, b1, b2, eps, (float)c1, (float)c2);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
    }
    if (loss) {
        std::vector<float> l((size_t)nb * mb_tiles, 0.f);
        TF_CUDA(c, cudaMemcpyAsync(l.data(), c->mlp_lossacc.p, sizeof(float) * l.size(), cudaMemcpyDeviceToHost, c->stream));
        TF_CUDA(c, cudaStreamSynchronize(c->stream));
        double s = 0.;
        for (int b = 0; b < nb; ++b) {
            const int cnt = (ntiles - b + nb - 1) / nb;
            for (int jj = 0; jj < cnt; ++jj) s += l[(size_t)b * mb_tiles + jj];
        }
        *loss = s / (2.0 * (double)n);
    }
    return mlp_err_check(c);
}

}  // namespace tf
