// Context plumbing, device-wide scans and kernel timing for libtracefem.
#include "tf_internal.cuh"

namespace tf {

int set_err(Context* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

TimedLaunch::TimedLaunch(Context* ctx, int kernel) : c(ctx), k(kernel) {
    if (c->timing) cudaEventRecord(c->ev0, c->stream);
}
TimedLaunch::~TimedLaunch() {
    if (c->timing) {
        cudaEventRecord(c->ev1, c->stream);
        cudaEventSynchronize(c->ev1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        c->timers[k].total_ms += ms;
        c->timers[k].launches += 1;
    }
}

// ---------------------------------------------------------------------------
// exclusive scan: tiles of kScanTile elements per block
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ T block_exclusive_scan(T v, T* smem_warp, T& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T x = v;
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < (kScanThreads / 32) ? smem_warp[lane] : T(0);
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < (kScanThreads / 32)) smem_warp[lane] = w;
    }
    __syncthreads();
    total = smem_warp[kScanThreads / 32 - 1];
    T before = warp > 0 ? smem_warp[warp - 1] : T(0);
    __syncthreads();
    return before + x - v;
}

__global__ void scan_tile_sums(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ tile_sums) {
    __shared__ int64_t sw[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
    for (int i = 0; i < kScanItems; ++i) {
        int64_t idx = base + (int64_t)i * kScanThreads + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    int64_t tot;
    block_exclusive_scan<int64_t>(s, sw, tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void scan_tile_offsets(int64_t* __restrict__ tile_sums, int64_t ntiles, int64_t* __restrict__ total) {
    __shared__ int64_t sw[kScanThreads / 32];
    int64_t carry = 0;
    for (int64_t b = 0; b < ntiles; b += kScanThreads) {
        int64_t idx = b + threadIdx.x;
        int64_t v = idx < ntiles ? tile_sums[idx] : 0;
        int64_t tot;
        int64_t ex = block_exclusive_scan<int64_t>(v, sw, tot);
        if (idx < ntiles) tile_sums[idx] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

template <class OutT>
__global__ void scan_tiles(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ tile_off,
                           const int64_t* __restrict__ total, OutT* __restrict__ out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = (OutT)(*total);
    if ((int64_t)blockIdx.x * kScanTile >= n) return;
    __shared__ int64_t sw[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems];
    int64_t s = 0;
    for (int i = 0; i < kScanItems; ++i) {
        int64_t idx = base + i;
        v[i] = idx < n ? in[idx] : 0;
        s += v[i];
    }
    int64_t tot;
    int64_t run = block_exclusive_scan<int64_t>(s, sw, tot) + tile_off[blockIdx.x];
    for (int i = 0; i < kScanItems; ++i) {
        int64_t idx = base + i;
        if (idx < n) out[idx] = (OutT)run;
        run += v[i];
    }
}

template <class OutT>
static int exclusive_scan_impl(Context* c, const int32_t* in, OutT* out, int64_t n, int64_t* total_host) {
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    TF_TRY(ensure(c, c->scan_tmp, (size_t)ntiles + 2));
    int64_t* tiles = c->scan_tmp.p;
    int64_t* total = tiles + ntiles + 1;
    if (ntiles > 0) {
        scan_tile_sums<<<(unsigned)ntiles, kScanThreads, 0, c->stream>>>(in, n, tiles);
        ++c->launches;
    }
    scan_tile_offsets<<<1, kScanThreads, 0, c->stream>>>(tiles, ntiles, total);
    ++c->launches;
    scan_tiles<OutT><<<(unsigned)(ntiles > 0 ? ntiles : 1), kScanThreads, 0, c->stream>>>(in, n, tiles, total, out);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    if (total_host) {
        TF_CUDA(c, cudaMemcpyAsync(total_host, total, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
        TF_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return TF_OK;
}

// out[0..n] with out[n] = total
int exclusive_scan_i32(Context* c, const int32_t* in, int64_t* out, int64_t n) {
    return exclusive_scan_impl<int64_t>(c, in, out, n, nullptr);
}
int exclusive_scan_i32_to_i32(Context* c, const int32_t* in, int32_t* out, int64_t n, int64_t* total) {
    int64_t tot = 0;
    TF_TRY(exclusive_scan_impl<int32_t>(c, in, out, n, &tot));
    if (tot > INT32_MAX) return set_err(c, TF_ERR_CAPACITY, "scan total exceeds int32 range");
    if (total) *total = tot;
    return TF_OK;
}

__global__ void k_fill_f64(double* p, int64_t n, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}

int fill_f64(Context* c, double* p, int64_t n, double v) {
    if (n <= 0) return TF_OK;
    k_fill_f64<<<grid_for(c, n), kBlock, 0, c->stream>>>(p, n, v);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    return TF_OK;
}

int sync_status(Context* c, int* status_out) {
    TF_CUDA(c, cudaMemcpyAsync(c->h_status, c->status.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    *status_out = c->h_status[0];
    return TF_OK;
}

}  // namespace tf
