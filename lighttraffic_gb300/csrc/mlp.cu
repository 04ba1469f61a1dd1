// mlp.cu -- kernels and host logic of the learned prefetcher.
//
// No counterpart in the reference, whose scheduler (src/Scheduler.h:84-171,
// :368-388) ranks partitions by the walkers waiting now; this policy runs the
// engine in waves and gives cache slots to the partitions a small network,
// trained online on the engine's own traces, predicts the most visits for.
//
// Kernels (FP32, deterministic reduction order):
//   mlp_forward  : one warp per row; lane j owns hidden units j and j+32,
//                  h = relu(x W1 + b1), y = h . W2 + b2 by a warp reduction;
//   mlp_backward : one CTA per hidden unit j; threads stride over rows and
//                  accumulate dL/dW1[:, j], dL/db1[j], dL/dW2[j] (and dL/db2,
//                  the loss in CTA 0), then a fixed-order tree reduction;
//                  L = mean (y - t)^2;
//   mlp_sgd      : v = mu v + g, w -= lr v;
//   pol_iter / pol_features / pol_labels / pol_demand: the policy's visit
//                  ring and moving average, feature rows, residual targets
//                  with the moving-average baseline loss, and forecasts.
#include "mlp.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace lt {

namespace {

constexpr int F = kMlpIn, H = kMlpHidden;
constexpr int kOffB1 = F * H, kOffW2 = F * H + H, kOffB2 = F * H + 2 * H;
constexpr int kBwdThreads = 256;

__global__ void mlp_forward(const float *__restrict__ x, uint32_t n, const float *__restrict__ p,
                            float *__restrict__ hbuf, float *__restrict__ y)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const float *xr = x + (uint64_t)warp * F;
    float a0 = p[kOffB1 + lane], a1 = p[kOffB1 + lane + 32];
#pragma unroll
    for (int i = 0; i < F; i++) {
        const float xi = xr[i];
        a0 = fmaf(xi, p[i * H + lane], a0);
        a1 = fmaf(xi, p[i * H + lane + 32], a1);
    }
    const float h0 = fmaxf(a0, 0.f), h1 = fmaxf(a1, 0.f);
    if (hbuf) {
        hbuf[(uint64_t)warp * H + lane] = h0;
        hbuf[(uint64_t)warp * H + lane + 32] = h1;
    }
    float s = h0 * p[kOffW2 + lane] + h1 * p[kOffW2 + lane + 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) y[warp] = s + p[kOffB2];
}

__device__ float block_sum(float v, float *sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = kBwdThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const float r = sh[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kBwdThreads) mlp_backward(const float *__restrict__ x, const float *__restrict__ t,
                                                            uint32_t n, const float *__restrict__ p,
                                                            const float *__restrict__ hbuf,
                                                            const float *__restrict__ y, float *__restrict__ grad,
                                                            float *__restrict__ loss)
{
    __shared__ float sh[kBwdThreads];
    const int j = blockIdx.x;
    const float w2 = p[kOffW2 + j];
    const float inv_n = 1.0f / (float)n;
    float gw1[F];
#pragma unroll
    for (int i = 0; i < F; i++) gw1[i] = 0.f;
    float gb1 = 0.f, gw2 = 0.f, gb2 = 0.f, l = 0.f;
    for (uint32_t r = threadIdx.x; r < n; r += kBwdThreads) {
        const float diff = y[r] - t[r];
        const float dy = 2.0f * diff * inv_n;
        const float h = hbuf[(uint64_t)r * H + j];
        gw2 = fmaf(dy, h, gw2);
        if (j == 0) {
            gb2 += dy;
            l = fmaf(diff, diff, l);
        }
        const float da = h > 0.f ? dy * w2 : 0.f;
        gb1 += da;
#pragma unroll
        for (int i = 0; i < F; i++) gw1[i] = fmaf(x[(uint64_t)r * F + i], da, gw1[i]);
    }
#pragma unroll
    for (int i = 0; i < F; i++) {
        const float s = block_sum(gw1[i], sh);
        if (threadIdx.x == 0) grad[i * H + j] = s;
    }
    const float sb1 = block_sum(gb1, sh);
    const float sw2 = block_sum(gw2, sh);
    if (threadIdx.x == 0) {
        grad[kOffB1 + j] = sb1;
        grad[kOffW2 + j] = sw2;
    }
    if (j == 0) {
        const float sb2 = block_sum(gb2, sh);
        const float sl = block_sum(l, sh);
        if (threadIdx.x == 0) {
            grad[kOffB2] = sb2;
            *loss = sl * inv_n;
        }
    }
}

__global__ void mlp_sgd(float *p, const float *g, float *m, float lr, float mu)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kMlpParams) {
        const float v = mu * m[i] + g[i];
        m[i] = v;
        p[i] -= lr * v;
    }
}

// splitmix64: initial weights only.
uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

Mlp::~Mlp()
{
    if (d_params_) cudaSetDevice(device_);
    for (float *q : {d_params_, d_grad_, d_mom_, d_x_, d_y_, d_pred_, d_h_, d_loss_})
        if (q) cudaFree(q);
    if (st_) cudaStreamDestroy(st_);
}

lt_status Mlp::init(int device, uint32_t max_rows, uint64_t seed)
{
    device_ = device;
    cap_ = max_rows ? max_rows : 1;
    LT_CUDA_TRY(cudaSetDevice(device));
    LT_CUDA_TRY(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
    LT_CUDA_TRY(cudaMalloc(&d_params_, 4 * kMlpParams));
    LT_CUDA_TRY(cudaMalloc(&d_grad_, 4 * kMlpParams));
    LT_CUDA_TRY(cudaMalloc(&d_mom_, 4 * kMlpParams));
    LT_CUDA_TRY(cudaMalloc(&d_x_, 4ull * cap_ * F));
    LT_CUDA_TRY(cudaMalloc(&d_y_, 4ull * cap_));
    LT_CUDA_TRY(cudaMalloc(&d_pred_, 4ull * cap_));
    LT_CUDA_TRY(cudaMalloc(&d_h_, 4ull * cap_ * H));
    LT_CUDA_TRY(cudaMalloc(&d_loss_, 4));
    LT_CUDA_TRY(cudaMemset(d_mom_, 0, 4 * kMlpParams));
    std::vector<float> w(kMlpParams, 0.f);
    uint64_t s = seed;
    const float a1 = std::sqrt(6.0f / (F + H)), a2 = std::sqrt(6.0f / (H + 1));
    for (int i = 0; i < F * H; i++) w[i] = a1 * (2.0f * (float)((splitmix(s) >> 40) * 0x1.0p-24) - 1.0f);
    for (int j = 0; j < H; j++) w[kOffW2 + j] = a2 * (2.0f * (float)((splitmix(s) >> 40) * 0x1.0p-24) - 1.0f);
    return set_params(w.data());
}

lt_status Mlp::set_params(const float *h)
{
    LT_CUDA_TRY(cudaMemcpy(d_params_, h, 4 * kMlpParams, cudaMemcpyHostToDevice));
    LT_CUDA_TRY(cudaMemset(d_mom_, 0, 4 * kMlpParams));
    return LT_OK;
}

lt_status Mlp::get_params(float *h)
{
    LT_CUDA_TRY(cudaMemcpy(h, d_params_, 4 * kMlpParams, cudaMemcpyDeviceToHost));
    return LT_OK;
}

namespace {

__global__ void copy_f32(float *__restrict__ dst, const float *__restrict__ src, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

// Device view of pinned, mapped host memory; null for other memory.
const float *mapped_view(const void *h)
{
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess || at.type != cudaMemoryTypeHost || !at.devicePointer) {
        cudaGetLastError();
        return nullptr;
    }
    return (const float *)at.devicePointer;
}

}  // namespace

// Host <-> device transfers of the network's rows.  Pinned, mapped buffers
// move by a copy kernel: copies on the copy engine would queue behind the
// partition loads of the engine that trains the network.
lt_status Mlp::move(float *dst, const float *src, uint64_t n, cudaMemcpyKind kind)
{
    const float *view = mapped_view(kind == cudaMemcpyHostToDevice ? (const void *)src : (const void *)dst);
    if (!view) {
        LT_CUDA_TRY(cudaMemcpyAsync(dst, src, 4ull * n, kind, st_));
        return LT_OK;
    }
    const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 152);
    if (kind == cudaMemcpyHostToDevice)
        copy_f32<<<blocks, 256, 0, st_>>>(dst, view, n);
    else
        copy_f32<<<blocks, 256, 0, st_>>>(const_cast<float *>(view), src, n);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

lt_status Mlp::upload(const float *h_x, const float *h_y, uint32_t n)
{
    if (n > cap_) return fail(LT_ERR_CAPACITY, "MLP batch of %u rows exceeds %u", n, cap_);
    LT_TRY(move(d_x_, h_x, (uint64_t)n * F, cudaMemcpyHostToDevice));
    if (h_y) LT_TRY(move(d_y_, h_y, n, cudaMemcpyHostToDevice));
    return LT_OK;
}

lt_status Mlp::forward(const float *h_x, uint32_t n, float *h_pred)
{
    if (n == 0) return LT_OK;
    LT_CUDA_TRY(cudaSetDevice(device_));
    LT_TRY(upload(h_x, nullptr, n));
    mlp_forward<<<(n * 32 + 255) / 256, 256, 0, st_>>>(d_x_, n, d_params_, nullptr, d_pred_);
    LT_CUDA_TRY(cudaGetLastError());
    LT_CUDA_TRY(cudaMemcpyAsync(h_pred, d_pred_, 4ull * n, cudaMemcpyDeviceToHost, st_));
    LT_CUDA_TRY(cudaStreamSynchronize(st_));
    return LT_OK;
}

lt_status Mlp::train(const float *h_x, const float *h_y, uint32_t n, float lr, float momentum, float *h_loss,
                     float *h_grad, float *h_pred)
{
    if (n == 0) return LT_OK;
    LT_CUDA_TRY(cudaSetDevice(device_));
    LT_TRY(upload(h_x, h_y, n));
    mlp_forward<<<(n * 32 + 255) / 256, 256, 0, st_>>>(d_x_, n, d_params_, d_h_, d_pred_);
    mlp_backward<<<H, kBwdThreads, 0, st_>>>(d_x_, d_y_, n, d_params_, d_h_, d_pred_, d_grad_, d_loss_);
    if (h_pred) LT_CUDA_TRY(cudaMemcpyAsync(h_pred, d_pred_, 4ull * n, cudaMemcpyDeviceToHost, st_));
    if (h_grad) LT_CUDA_TRY(cudaMemcpyAsync(h_grad, d_grad_, 4 * kMlpParams, cudaMemcpyDeviceToHost, st_));
    if (lr > 0.f) mlp_sgd<<<(kMlpParams + 255) / 256, 256, 0, st_>>>(d_params_, d_grad_, d_mom_, lr, momentum);
    LT_CUDA_TRY(cudaGetLastError());
    if (h_loss) LT_CUDA_TRY(cudaMemcpyAsync(h_loss, d_loss_, 4, cudaMemcpyDeviceToHost, st_));
    LT_CUDA_TRY(cudaStreamSynchronize(st_));
    return LT_OK;
}

lt_status Mlp::train_dev(const float *d_x, const float *d_y, uint32_t n, float lr, float momentum, float *d_loss)
{
    if (n > cap_) return fail(LT_ERR_CAPACITY, "MLP batch of %u rows exceeds %u", n, cap_);
    mlp_forward<<<(n * 32 + 255) / 256, 256, 0, st_>>>(d_x, n, d_params_, d_h_, d_pred_);
    mlp_backward<<<H, kBwdThreads, 0, st_>>>(d_x, d_y, n, d_params_, d_h_, d_pred_, d_grad_, d_loss);
    mlp_sgd<<<(kMlpParams + 255) / 256, 256, 0, st_>>>(d_params_, d_grad_, d_mom_, lr, momentum);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

lt_status Mlp::forward_dev(const float *d_x, uint32_t n, float *d_pred)
{
    if (n > cap_) return fail(LT_ERR_CAPACITY, "MLP batch of %u rows exceeds %u", n, cap_);
    mlp_forward<<<(n * 32 + 255) / 256, 256, 0, st_>>>(d_x, n, d_params_, nullptr, d_pred);
    LT_CUDA_TRY(cudaGetLastError());
    return LT_OK;
}

lt_status Mlp::record(cudaEvent_t ev)
{
    LT_CUDA_TRY(cudaEventRecord(ev, st_));
    return LT_OK;
}

// ------------------------------------------------------------ the policy

namespace {

constexpr int kHist = 8;
constexpr int kEvery = 2;  // features, training and prediction every kEvery iterations
constexpr float kLearningRate = 0.02f;
constexpr float kMomentum = 0.9f;
constexpr float kEmaKeep = 0.95f;
constexpr int kRunWarm = 16;      // iterations of a run before its own forecast drives the cache
constexpr double kGateKeep = 0.8;  // running average of the validation losses the gate compares
constexpr int kRing = kHist + kLabelHorizon + 1;    // visit history ring (iterations)
constexpr int kSnaps = kLabelHorizon / kEvery + 2;  // feature snapshots awaiting labels
constexpr int kStage = 4;                           // host staging slots (iterations in flight)

// ---- device side of the policy: features, labels and forecasts.  The host
// stages per iteration the visits of every partition (u32) and, every kEvery
// iterations, its waiting walkers, residency and iterations since last use
// (f32); everything else lives on the device.

// ring[slot] = visits; ema = kEmaKeep ema + (1 - kEmaKeep) visits.
__global__ void pol_iter(uint32_t *ring, float *ema, const uint32_t *visits, uint32_t P, uint32_t slot)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const uint32_t v = visits[p];
        ring[(uint64_t)slot * P + p] = v;
        ema[p] = kEmaKeep * ema[p] + (1.0f - kEmaKeep) * (float)v;
    }
}

// Feature rows of iteration t (layout in mlp.h).  dyn = waiting | resident | gap.
__global__ void pol_features(float *X, const uint32_t *ring, const float *ema, const float *stat, const float *dyn,
                             uint32_t P, uint64_t t)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        float *x = X + (uint64_t)p * kMlpIn;
        x[0] = log1pf(dyn[p]) / 16.0f;
        for (int k = 0; k < kHist; k++)
            x[1 + k] = (uint64_t)k < t ? log1pf((float)ring[(uint64_t)((t - k) % kRing) * P + p]) / 16.0f : 0.0f;
        x[9] = stat[p];
        x[10] = stat[P + p];
        x[11] = dyn[P + p];
        x[12] = log1pf(dyn[2 * P + p]) / 16.0f;
        x[13] = log1pf(ema[p]) / 16.0f;
        x[14] = (float)p / (float)P;
        x[15] = log1pf(ema[p] * (float)kLabelHorizon) / 16.0f;  // moving-average forecast
    }
}

// Targets for the snapshot taken kLabelHorizon iterations before t: the
// visits since then, as a correction to the snapshot's moving-average
// forecast; base = the mean squared error of that forecast alone (one CTA,
// fixed reduction order).
__global__ void __launch_bounds__(256) pol_labels(float *Y, float *base, const float *Xold, const uint32_t *ring,
                                                  uint32_t P, uint64_t t)
{
    __shared__ float sh[256];
    float acc = 0.f;
    for (uint32_t p = threadIdx.x; p < P; p += 256) {
        float sum = 0.f;
        for (int k = 0; k < kLabelHorizon; k++) sum += (float)ring[(uint64_t)((t - k) % kRing) * P + p];
        const float y = log1pf(sum) / 16.0f - Xold[(uint64_t)p * kMlpIn + 15];
        Y[p] = y;
        acc = fmaf(y, y, acc);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *base = sh[0] / (float)P;
}

// demand = visits over the label horizon as the network predicts them;
// base_demand = the same from the moving-average forecast alone.
__global__ void pol_demand(float *demand, float *base_demand, const float *pred, const float *X, uint32_t P)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const float f = X[(uint64_t)p * kMlpIn + 15];
        demand[p] = expm1f(fmaxf(0.f, f + pred[p]) * 16.0f);
        base_demand[p] = expm1f(fmaxf(0.f, f) * 16.0f);
    }
}

__global__ void pol_copy(float *dst, const float *src, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// Eviction scores are predicted visits (walkers entering the partition,
// cached or not) over the next kLabelHorizon iterations plus the walkers
// already waiting.  The network runs on its own stream; the host stages a few
// kilobytes per iteration and picks up the forecasts of the previous pass
// when they are ready, never waiting for them.
class LearnedPolicy : public Policy {
public:
    // use_net = false: the same decisions from a moving average of visits
    // instead of the network (the ablation baseline), kept on the host.
    LearnedPolicy(const lt_graph &g, bool use_net) : P_(g.P()), use_net_(use_net)
    {
        static_mass_.resize(P_);
        history_.assign(P_, 0.0);
        run_visits_.assign(P_, 0.0);
        for (uint32_t p = 0; p < P_; p++) static_mass_[p] = g.edge_off[p + 1] - g.edge_off[p];
        ema_.assign(P_, 0.f);
        demand_.assign(P_, 0.0);
        snap_t_.assign(kSnaps, 0);
        stat_.resize(2ull * P_);
        for (uint32_t p = 0; p < P_; p++) {
            stat_[p] = std::log1p((float)(g.edge_off[p + 1] - g.edge_off[p])) / 24.0f;
            stat_[P_ + p] = std::log1p((float)(g.node_off[p + 1] - g.node_off[p])) / 24.0f;
        }
    }

    ~LearnedPolicy() override
    {
        if (ev_) cudaEventDestroy(ev_);
        for (cudaEvent_t e : stage_ev_)
            if (e) cudaEventDestroy(e);
        for (void *q : {(void *)d_ring_, (void *)d_ema_, (void *)d_stat_, (void *)d_X_, (void *)d_Y_, (void *)d_out_,
                        (void *)d_pred_})
            if (q) cudaFree(q);
        host_free(h_stage_);
        host_free(h_out_);
    }

    lt_status init(int device)
    {
        if (!use_net_) return LT_OK;
        LT_TRY(net_.init(device, P_, 0x5EEDull));
        // the network learns a correction to the moving-average forecast:
        // a zero output layer starts it exactly at that forecast
        std::vector<float> w(kMlpParams);
        LT_TRY(net_.get_params(w.data()));
        for (int j = 0; j <= kMlpHidden; j++) w[kMlpIn * kMlpHidden + kMlpHidden + j] = 0.f;
        LT_TRY(net_.set_params(w.data()));
        LT_CUDA_TRY(cudaMalloc(&d_ring_, 4ull * kRing * P_));
        LT_CUDA_TRY(cudaMalloc(&d_ema_, 4ull * P_));
        LT_CUDA_TRY(cudaMalloc(&d_stat_, 8ull * P_));
        LT_CUDA_TRY(cudaMalloc(&d_X_, 4ull * kSnaps * P_ * kMlpIn));
        LT_CUDA_TRY(cudaMalloc(&d_Y_, 4ull * P_));
        LT_CUDA_TRY(cudaMalloc(&d_out_, 4ull * (2 * P_ + 2)));
        LT_CUDA_TRY(cudaMalloc(&d_pred_, 4ull * P_));
        LT_CUDA_TRY(cudaMemset(d_ring_, 0, 4ull * kRing * P_));
        LT_CUDA_TRY(cudaMemset(d_ema_, 0, 4ull * P_));
        LT_CUDA_TRY(cudaMemset(d_out_, 0, 4ull * (2 * P_ + 2)));
        LT_CUDA_TRY(cudaMemcpy(d_stat_, stat_.data(), 8ull * P_, cudaMemcpyHostToDevice));
        LT_TRY(host_alloc(h_stage_, 16ull * P_ * kStage, true));
        LT_TRY(host_alloc(h_out_, 4ull * (2 * P_ + 2), true));
        if (!h_stage_.pinned || !h_out_.pinned) return fail(LT_ERR_NOMEM, "pinned staging for the prefetcher");
        void *dv = nullptr;
        LT_CUDA_TRY(cudaHostGetDevicePointer(&dv, h_stage_.ptr, 0));
        stage_dev_ = (uint8_t *)dv;
        LT_CUDA_TRY(cudaHostGetDevicePointer(&dv, h_out_.ptr, 0));
        out_dev_ = (float *)dv;
        LT_CUDA_TRY(cudaEventCreateWithFlags(&ev_, cudaEventDisableTiming));
        for (cudaEvent_t &e : stage_ev_) LT_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        return LT_OK;
    }

    // Memory across runs: the entries each partition drew in the previous
    // runs (each run halves the weight of the ones before).  Until this run
    // has trained the forecast (kRunWarm iterations), cache slots go to the
    // partitions that drew the most -- on c2 the best fixed set of 212
    // partitions catches 23 % of the entries, the first-come fill 16 %.
    void run_start() override
    {
        double sum = 0;
        for (uint32_t p = 0; p < P_; p++) sum += run_visits_[p];
        if (sum > 0) {
            for (uint32_t p = 0; p < P_; p++) history_[p] = 0.5 * history_[p] + run_visits_[p];
            have_history_ = true;
        }
        std::fill(run_visits_.begin(), run_visits_.end(), 0.0);
        t_run_ = 0;
    }

    void observe(const SchedView &v) override
    {
        t_++;
        t_run_++;
        for (uint32_t p = 0; p < P_; p++) run_visits_[p] += v.visits[p];
        if (!use_net_) {
            for (uint32_t p = 0; p < P_; p++) ema_[p] = kEmaKeep * ema_[p] + (1.0f - kEmaKeep) * (float)v.visits[p];
            if (t_ % kEvery) return;
            for (uint32_t p = 0; p < P_; p++) demand_[p] = (double)ema_[p] * kLabelHorizon;
            ready_ = t_ >= (uint64_t)kLabelHorizon;
            return;
        }
        if (failed_) return;
        // stage this iteration's visits (slot reused kStage iterations later)
        const int slot = (int)(t_ % kStage);
        if (cudaEventSynchronize(stage_ev_[slot]) != cudaSuccess) return fail_net();
        uint8_t *stage = (uint8_t *)h_stage_.ptr + 16ull * P_ * slot;
        const uint8_t *stage_dev = stage_dev_ + 16ull * P_ * slot;
        std::memcpy(stage, v.visits, 4ull * P_);
        cudaStream_t st = net_.stream();
        const unsigned blocks = (P_ + 255) / 256;
        pol_iter<<<blocks, 256, 0, st>>>(d_ring_, d_ema_, (const uint32_t *)stage_dev, P_, (uint32_t)(t_ % kRing));
        if (t_ % kEvery) {
            if (cudaEventRecord(stage_ev_[slot], st) != cudaSuccess) fail_net();
            return;
        }
        // pick up the previous prediction pass if it has finished; never wait for it
        if (inflight_) {
            if (cudaEventQuery(ev_) != cudaSuccess) {
                cudaGetLastError();
                skipped_++;
                if (cudaEventRecord(stage_ev_[slot], st) != cudaSuccess) fail_net();
                return;
            }
            inflight_ = false;
            const float *out = (const float *)h_out_.ptr;
            if (train_enqueued_) {
                losses_.push_back({out[P_], out[P_ + 1]});
                // running validation of the network against the moving
                // average it corrects (each loss is taken before the SGD
                // step on that batch, i.e. on data not yet trained on)
                net_avg_ = kGateKeep * net_avg_ + (1.0 - kGateKeep) * out[P_];
                base_avg_ = kGateKeep * base_avg_ + (1.0 - kGateKeep) * out[P_ + 1];
                train_enqueued_ = false;
            }
            if (pred_enqueued_) {
                // act on the network only while it forecasts better than
                // the moving average; otherwise on the moving average
                const bool net = net_avg_ < base_avg_;
                const float *src = net ? out : out + P_ + 2;
                for (uint32_t p = 0; p < P_; p++) demand_[p] = src[p];
                pred_enqueued_ = false;
                ready_ = true;
                predictions_++;
                net_used_ += net;
            }
        }
        float *dyn = (float *)(stage + 4ull * P_);
        for (uint32_t p = 0; p < P_; p++) {
            dyn[p] = (float)v.waiting[p];
            dyn[P_ + p] = v.slot_of[p] >= 0 ? 1.0f : 0.0f;
            dyn[2 * P_ + p] = (float)(v.iteration - std::min<uint64_t>(v.iteration, v.last_used[p]));
        }
        const int s = (int)((t_ / kEvery) % kSnaps);
        float *Xs = d_X_ + (uint64_t)s * P_ * kMlpIn;
        pol_features<<<blocks, 256, 0, st>>>(Xs, d_ring_, d_ema_, d_stat_, (const float *)(stage_dev + 4ull * P_), P_,
                                             t_);
        snap_t_[s] = t_;
        // train on the snapshot whose label horizon has passed
        const int old = (int)(((t_ / kEvery) + kSnaps - (kLabelHorizon / kEvery)) % kSnaps);
        if (t_ >= (uint64_t)kLabelHorizon + kEvery && snap_t_[old] + kLabelHorizon == t_) {
            const float *Xo = d_X_ + (uint64_t)old * P_ * kMlpIn;
            pol_labels<<<1, 256, 0, st>>>(d_Y_, d_out_ + P_ + 1, Xo, d_ring_, P_, t_);
            if (net_.train_dev(Xo, d_Y_, P_, kLearningRate, kMomentum, d_out_ + P_) != LT_OK) return fail_net();
            trained_++;
            train_enqueued_ = true;
        }
        if (trained_ >= 4) {
            if (net_.forward_dev(Xs, P_, d_pred_) != LT_OK) return fail_net();
            pol_demand<<<blocks, 256, 0, st>>>(d_out_, d_out_ + P_ + 2, d_pred_, Xs, P_);
            pred_enqueued_ = true;
        }
        pol_copy<<<(2 * P_ + 2 + 255) / 256, 256, 0, st>>>(out_dev_, d_out_, 2 * P_ + 2);
        if (cudaEventRecord(ev_, st) != cudaSuccess || cudaEventRecord(stage_ev_[slot], st) != cudaSuccess)
            return fail_net();
        inflight_ = true;
    }

    const char *name() const override { return use_net_ ? "learned" : "frequency"; }

    bool wave() const override { return true; }

    void stats(lt_policy_stats &st) const override
    {
        Policy::stats(st);
        st.train_steps = trained_;
        st.predictions = predictions_;
        // second half of the batches: after the network has had time to learn
        const size_t from = losses_.size() / 2;
        double a = 0, b = 0;
        for (size_t i = from; i < losses_.size(); i++) {
            a += losses_[i].first;
            b += losses_[i].second;
        }
        const size_t n = losses_.size() - from;
        st.net_loss = n ? a / n : 0.0;
        st.baseline_loss = n ? b / n : 0.0;
        st.net_used = net_used_;
    }

    // Predicted visits once the predictor is trained; before that, the
    // partition's edge count (a hub-heavy RMAT prior).
    // The partitions that drew the most entries in the previous runs.
    bool prefill(const SchedView &v, std::vector<uint32_t> &order) override
    {
        if (!have_history_ || t_run_ > 0) return false;
        order.resize(P_);
        for (uint32_t p = 0; p < P_; p++) order[p] = p;
        std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
            return history_[a] != history_[b] ? history_[a] > history_[b] : a < b;
        });
        return true;
    }

    double cache_score(const SchedView &v, uint32_t p) override
    {
        if (have_history_ && t_run_ < (uint64_t)kRunWarm) return history_[p] + (double)v.waiting[p];
        return ready_ ? demand_[p] + (double)v.waiting[p] : (double)static_mass_[p];
    }

    // Forecast entries per iteration: the network's (learned) or the moving
    // average's (frequency) prediction over the label horizon, per iteration.
    double visit_rate(const SchedView &, uint32_t p) override
    {
        return ready_ && t_run_ >= (uint64_t)kRunWarm ? demand_[p] / (double)kLabelHorizon : -1.0;
    }

private:

    // A CUDA error in the policy's own work: keep the last forecasts and stop
    // training (scheduling decisions never affect results).
    void fail_net()
    {
        cudaGetLastError();
        failed_ = true;
    }

    uint32_t P_;
    bool use_net_;
    Mlp net_;
    uint64_t t_ = 0, trained_ = 0, skipped_ = 0, predictions_ = 0, net_used_ = 0, t_run_ = 0;
    std::vector<double> history_, run_visits_;  // entries per partition: previous runs (decayed), this run
    bool have_history_ = false;
    double net_avg_ = 1e30, base_avg_ = 0.0;  // validation gate (running losses)
    bool ready_ = false, inflight_ = false, pred_enqueued_ = false, train_enqueued_ = false, failed_ = false;
    std::vector<std::pair<double, double>> losses_;  // (network, moving average) per training batch
    cudaEvent_t ev_ = nullptr;
    cudaEvent_t stage_ev_[kStage] = {};
    HostBuf h_stage_, h_out_;
    uint8_t *stage_dev_ = nullptr;
    float *out_dev_ = nullptr;
    uint32_t *d_ring_ = nullptr;
    float *d_ema_ = nullptr, *d_stat_ = nullptr, *d_X_ = nullptr, *d_Y_ = nullptr, *d_out_ = nullptr, *d_pred_ = nullptr;
    std::vector<uint64_t> snap_t_, static_mass_;
    std::vector<float> ema_, stat_;
    std::vector<double> demand_;
};

}  // namespace

lt_status make_learned_policy(const lt_graph &g, int device, bool use_net, Policy **out)
{
    LearnedPolicy *p = new LearnedPolicy(g, use_net);
    lt_status s = p->init(device);
    if (s != LT_OK) {
        delete p;
        return s;
    }
    *out = p;
    return LT_OK;
}

}  // namespace lt

// Test entry point: forward + backward (and optionally one SGD step) of the
// prefetcher network on caller data.  No counterpart in the reference.
extern "C" lt_status lt_mlp_check(int device, uint32_t n, const float *x, const float *y, const float *params,
                                  float lr, float momentum, float *pred_out, float *grad_out, float *loss_out,
                                  float *params_out)
{
    if (!x || !y || !params || n == 0) return lt::fail(LT_ERR_INVALID, "null or empty argument");
    lt::Mlp m;
    LT_TRY(m.init(device, n, 1));
    LT_TRY(m.set_params(params));
    LT_TRY(m.train(x, y, n, lr, momentum, loss_out, grad_out, pred_out));
    if (params_out) LT_TRY(m.get_params(params_out));
    return LT_OK;
}
