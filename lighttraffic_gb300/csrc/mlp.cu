// mlp.cu -- kernels and host logic of the learned prefetcher.
//
// No counterpart in the reference, whose scheduler (src/Scheduler.h:84-171,
// :368-388) ranks partitions by the walkers waiting now; this policy ranks
// them by the arrivals a small network predicts from the engine's own traces,
// and loads the predicted partitions ahead of need.
//
// Kernels (FP32, deterministic reduction order):
//   mlp_forward  : one warp per row; lane j owns hidden units j and j+32,
//                  h = relu(x W1 + b1), y = h . W2 + b2 by a warp reduction;
//   mlp_backward : one CTA per hidden unit j; threads stride over rows and
//                  accumulate dL/dW1[:, j], dL/db1[j], dL/dW2[j] (and dL/db2,
//                  the loss in CTA 0), then a fixed-order tree reduction;
//                  L = mean (y - t)^2;
//   mlp_sgd      : v = mu v + g, w -= lr v.
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

lt_status Mlp::upload(const float *h_x, const float *h_y, uint32_t n)
{
    if (n > cap_) return fail(LT_ERR_CAPACITY, "MLP batch of %u rows exceeds %u", n, cap_);
    LT_CUDA_TRY(cudaMemcpyAsync(d_x_, h_x, 4ull * n * F, cudaMemcpyHostToDevice, st_));
    if (h_y) LT_CUDA_TRY(cudaMemcpyAsync(d_y_, h_y, 4ull * n, cudaMemcpyHostToDevice, st_));
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

lt_status Mlp::train_async(const float *h_x, const float *h_y, uint32_t n, float lr, float momentum, float *h_loss)
{
    LT_CUDA_TRY(cudaSetDevice(device_));
    LT_TRY(upload(h_x, h_y, n));
    mlp_forward<<<(n * 32 + 255) / 256, 256, 0, st_>>>(d_x_, n, d_params_, d_h_, d_pred_);
    mlp_backward<<<H, kBwdThreads, 0, st_>>>(d_x_, d_y_, n, d_params_, d_h_, d_pred_, d_grad_, d_loss_);
    mlp_sgd<<<(kMlpParams + 255) / 256, 256, 0, st_>>>(d_params_, d_grad_, d_mom_, lr, momentum);
    LT_CUDA_TRY(cudaGetLastError());
    if (h_loss) LT_CUDA_TRY(cudaMemcpyAsync(h_loss, d_loss_, 4, cudaMemcpyDeviceToHost, st_));
    return LT_OK;
}

lt_status Mlp::forward_async(const float *h_x, uint32_t n, float *h_pred)
{
    LT_CUDA_TRY(cudaSetDevice(device_));
    LT_TRY(upload(h_x, nullptr, n));
    mlp_forward<<<(n * 32 + 255) / 256, 256, 0, st_>>>(d_x_, n, d_params_, nullptr, d_pred_);
    LT_CUDA_TRY(cudaGetLastError());
    LT_CUDA_TRY(cudaMemcpyAsync(h_pred, d_pred_, 4ull * n, cudaMemcpyDeviceToHost, st_));
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
constexpr int kEvery = 8;  // features, training and prediction every kEvery iterations
constexpr float kLearningRate = 0.02f;
constexpr float kMomentum = 0.9f;
constexpr int kRing = kHist + kLabelHorizon + 1;    // visit history ring (iterations)
constexpr int kSnaps = kLabelHorizon / kEvery + 2;  // feature snapshots awaiting labels

// Scores are predicted visits (walkers entering the partition, cached or not)
// over the next kLabelHorizon iterations plus the walkers already waiting.
// Cache decisions only trade a cached partition for one predicted clearly
// busier (twice the score plus the zero-copy threshold), so noise in the
// predictions does not turn into load / evict churn.
class LearnedPolicy : public Policy {
public:
    // use_net = false: the same decisions from a moving average of visits
    // instead of the network (the ablation baseline).
    LearnedPolicy(const lt_graph &g, bool use_net) : P_(g.P()), use_net_(use_net)
    {
        edge_feat_.resize(P_);
        node_feat_.resize(P_);
        static_mass_.resize(P_);
        for (uint32_t p = 0; p < P_; p++) {
            static_mass_[p] = g.edge_off[p + 1] - g.edge_off[p];
            edge_feat_[p] = std::log1p((float)(g.edge_off[p + 1] - g.edge_off[p])) / 24.0f;
            node_feat_[p] = std::log1p((float)(g.node_off[p + 1] - g.node_off[p])) / 24.0f;
        }
        ring_.assign((size_t)kRing * P_, 0u);
        ema_.assign(P_, 0.f);
        demand_.assign(P_, 0.0);
        snap_t_.assign(kSnaps, 0);
    }

    ~LearnedPolicy() override
    {
        if (ev_) cudaEventDestroy(ev_);
        host_free(h_loss_);
        host_free(h_x_);
        host_free(h_y_);
        host_free(h_pred_);
    }

    lt_status init(int device)
    {
        if (!use_net_) return LT_OK;
        LT_TRY(net_.init(device, P_, 0x5EEDull));
        LT_TRY(host_alloc(h_x_, 4ull * kSnaps * P_ * kMlpIn, true));
        LT_TRY(host_alloc(h_y_, 4ull * P_, true));
        LT_TRY(host_alloc(h_pred_, 4ull * P_, true));
        LT_TRY(host_alloc(h_loss_, 16, true));
        LT_CUDA_TRY(cudaEventCreateWithFlags(&ev_, cudaEventDisableTiming));
        return LT_OK;
    }

    int32_t victim(const SchedView &v, int32_t except, uint32_t incoming) override
    {
        if (!ready_) return Policy::victim(v, except, incoming);
        int32_t best = -1;
        for (uint32_t i = 0; i < v.P; i++) {
            if (v.slot_of[i] < 0 || (int32_t)i == except || i == incoming) continue;
            if (best < 0 || score(v, i) < score(v, best) ||
                (score(v, i) == score(v, best) && v.last_used[i] < v.last_used[best]))
                best = (int32_t)i;
        }
        return best;
    }

    // Zero-copy follows the reference threshold on waiting walkers.

    // Look-ahead: while p computes, load the non-cached partitions with the
    // most waiting walkers, but only into slots whose partitions are
    // predicted to be far less busy.
    void prefetch_order(const SchedView &v, uint32_t exclude, std::vector<uint32_t> &out) override
    {
        out.clear();
        if (!ready_) return;
        for (uint32_t i = 0; i < v.P; i++)
            if (i != exclude && v.slot_of[i] < 0 && v.waiting[i] >= v.zc_threshold) out.push_back(i);
        const size_t k = std::min<size_t>(out.size(), 4);
        std::partial_sort(out.begin(), out.begin() + k, out.end(), [&](uint32_t a, uint32_t b) {
            return v.waiting[a] != v.waiting[b] ? v.waiting[a] > v.waiting[b] : a < b;
        });
        out.resize(k);
    }

    // Look-ahead loads measured as a net loss on the 2^33-edge graph (each one
    // displaced a partition that was needed again); kept available, off.
    size_t prefetch_depth(const SchedView &) override { return 0; }

    int32_t victim_for_prefetch(const SchedView &v, int32_t computing, uint32_t c) override
    {
        const int32_t w = victim(v, computing, c);
        if (w < 0) return -1;
        return score(v, c) > 4.0 * score(v, (uint32_t)w) + (double)v.zc_threshold ? w : -1;
    }

    void observe(const SchedView &v) override
    {
        t_++;
        std::memcpy(&ring_[(size_t)(t_ % kRing) * P_], v.visits, 4ull * P_);
        for (uint32_t p = 0; p < P_; p++) ema_[p] = 0.95f * ema_[p] + 0.05f * (float)v.visits[p];
        if (t_ % kEvery) return;
        if (!use_net_) {
            for (uint32_t p = 0; p < P_; p++) demand_[p] = (double)ema_[p] * kLabelHorizon;
            ready_ = t_ >= (uint64_t)kLabelHorizon;
            return;
        }
        // the work enqueued kEvery iterations ago has long finished: take its
        // predictions, and its host buffers are free again
        if (inflight_) {
            cudaEventSynchronize(ev_);
            inflight_ = false;
            if (train_enqueued_) {
                losses_.push_back({*(const float *)h_loss_.ptr, pending_baseline_});
                train_enqueued_ = false;
            }
            if (pred_enqueued_) {
                const float *pred = (const float *)h_pred_.ptr;
                for (uint32_t p = 0; p < P_; p++) demand_[p] = std::expm1(std::max(0.f, pred[p]) * 16.0f);
                pred_enqueued_ = false;
                ready_ = true;
                predictions_++;
            }
        }
        const int s = (int)((t_ / kEvery) % kSnaps);
        float *xs = (float *)h_x_.ptr + (size_t)s * P_ * kMlpIn;
        features(v, xs);
        snap_t_[s] = t_;
        // train on the snapshot whose label horizon has passed
        const int old = (int)(((t_ / kEvery) + kSnaps - (kLabelHorizon / kEvery)) % kSnaps);
        bool enq = false;
        if (t_ >= (uint64_t)kLabelHorizon + kEvery && snap_t_[old] + kLabelHorizon == t_) {
            float *y = (float *)h_y_.ptr;
            for (uint32_t p = 0; p < P_; p++) {
                float sum = 0.f;
                for (int k = 0; k < kLabelHorizon; k++) sum += (float)ring_[(size_t)((t_ - k) % kRing) * P_ + p];
                y[p] = std::log1p(sum) / 16.0f;
            }
            const float *xo = (const float *)h_x_.ptr + (size_t)old * P_ * kMlpIn;
            // the predictor the network replaces: the visit moving average of
            // the snapshot, scaled to the label horizon
            double base = 0.0;
            for (uint32_t p = 0; p < P_; p++) {
                const float ema = std::expm1(xo[(size_t)p * kMlpIn + 13] * 16.0f);
                const float yb = std::log1p(ema * (float)kLabelHorizon) / 16.0f;
                base += (double)(yb - y[p]) * (yb - y[p]);
            }
            pending_baseline_ = base / P_;
            if (net_.train_async(xo, y, P_, kLearningRate, kMomentum, (float *)h_loss_.ptr) == LT_OK) {
                trained_++;
                train_enqueued_ = true;
                enq = true;
            }
        }
        if (trained_ >= 4 && net_.forward_async(xs, P_, (float *)h_pred_.ptr) == LT_OK) {
            pred_enqueued_ = true;
            enq = true;
        }
        if (enq && net_.record(ev_) == LT_OK) inflight_ = true;
        cudaGetLastError();
    }

    const char *name() const override { return use_net_ ? "learned" : "frequency"; }

    bool single_pass() const override { return false; }
    // Serving keeps few walkers in flight, so reading cold partitions zero-copy
    // costs little and lets every admitted query finish in one step; the
    // network then chooses which partitions hold cache slots.
    bool serve_single_pass() const override { return true; }

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
    }

    // Few walkers per batch make single scores noisy: swap rarely and only for
    // a clearly hotter partition, so the cache settles on the hot set.
    size_t swap_budget() const override { return 4; }
    double swap_ratio() const override { return 4.0; }
    // Predicted visits once the predictor is trained; before that, the
    // partition's edge count (a hub-heavy RMAT prior).
    double cache_score(const SchedView &v, uint32_t p) override
    {
        return ready_ ? demand_[p] + (double)v.waiting[p] : (double)static_mass_[p];
    }

private:
    double score(const SchedView &v, uint32_t p) const { return (double)v.waiting[p] + demand_[p]; }

    float hist(uint32_t p, int k) const
    {
        if ((uint64_t)k >= t_) return 0.f;
        return std::log1p((float)ring_[(size_t)((t_ - k) % kRing) * P_ + p]) / 16.0f;
    }

    void features(const SchedView &v, float *xs) const
    {
        for (uint32_t p = 0; p < P_; p++) {
            float *x = xs + (size_t)p * kMlpIn;
            x[0] = std::log1p((float)v.waiting[p]) / 16.0f;
            for (int k = 0; k < kHist; k++) x[1 + k] = hist(p, k);
            x[9] = edge_feat_[p];
            x[10] = node_feat_[p];
            x[11] = v.slot_of[p] >= 0 ? 1.0f : 0.0f;
            x[12] = std::log1p((float)(v.iteration - std::min<uint64_t>(v.iteration, v.last_used[p]))) / 16.0f;
            x[13] = std::log1p(ema_[p]) / 16.0f;
            x[14] = (float)p / (float)P_;
            x[15] = 0.0f;
        }
    }

    uint32_t P_;
    bool use_net_;
    Mlp net_;
    uint64_t t_ = 0, trained_ = 0;
    bool ready_ = false, inflight_ = false, pred_enqueued_ = false, train_enqueued_ = false;
    double pending_baseline_ = 0.0;
    uint64_t predictions_ = 0;
    std::vector<std::pair<double, double>> losses_;  // (network, moving average) per training batch
    HostBuf h_loss_;
    cudaEvent_t ev_ = nullptr;
    HostBuf h_x_, h_y_, h_pred_;
    std::vector<uint32_t> ring_;
    std::vector<uint64_t> snap_t_, static_mass_;
    std::vector<float> edge_feat_, node_feat_, ema_;
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
