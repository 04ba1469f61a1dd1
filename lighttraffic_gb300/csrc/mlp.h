// mlp.h -- the learned prefetcher: a 2-layer FP32 MLP (kMlpIn inputs, kMlpHidden
// ReLU units, 1 output) trained online on the GPU by hand-written forward,
// backward and SGD kernels, and the scheduling policy that uses it.
//
// The network predicts, per partition, log1p(walkers entering it over the
// next kLabelHorizon iterations) / 16 as a correction to the moving-average
// forecast (its output layer starts at zero, so it starts at that forecast)
// from: waiting walkers, the visits of the last 8 iterations, a visit moving
// average and its forecast, the partition's edge and vertex mass, its
// residency bit, the iterations since it was last used and its position in
// the vertex order.  It is trained on the engine's own traces: every
// iteration's features are kept until their label (the visits that follow)
// is known.
#pragma once

#include <cstdint>

#include "common.h"
#include "graph.h"
#include "sched.h"

namespace lt {

constexpr int kMlpIn = 16;
constexpr int kMlpHidden = 64;
constexpr int kMlpParams = kMlpIn * kMlpHidden + kMlpHidden + kMlpHidden + 1;  // W1 | b1 | W2 | b2
constexpr int kLabelHorizon = 8;

// Device-resident network.
class Mlp {
public:
    ~Mlp();
    lt_status init(int device, uint32_t max_rows, uint64_t seed);
    // Upload host weights (kMlpParams floats, layout W1[i*H+j] | b1 | W2 | b2).
    lt_status set_params(const float *h_params);
    lt_status get_params(float *h_params);
    // pred[n] = f(x[n*kMlpIn])
    lt_status forward(const float *h_x, uint32_t n, float *h_pred);
    // Forward + backward of the mean squared error on (x, y); gradients in the
    // parameter layout; applies SGD with momentum when lr > 0.
    lt_status train(const float *h_x, const float *h_y, uint32_t n, float lr, float momentum, float *h_loss,
                    float *h_grad, float *h_pred);
    // Device-resident rows, enqueued on stream() without waiting: one SGD
    // step on (d_x, d_y) writing the pre-step loss to d_loss, and a forward.
    lt_status train_dev(const float *d_x, const float *d_y, uint32_t n, float lr, float momentum, float *d_loss);
    lt_status forward_dev(const float *d_x, uint32_t n, float *d_pred);
    cudaStream_t stream() const { return st_; }
    lt_status record(cudaEvent_t ev);

private:
    int device_ = 0;
    uint32_t cap_ = 0;
    cudaStream_t st_ = nullptr;
    float *d_params_ = nullptr, *d_grad_ = nullptr, *d_mom_ = nullptr;
    float *d_x_ = nullptr, *d_y_ = nullptr, *d_pred_ = nullptr, *d_h_ = nullptr, *d_loss_ = nullptr;
    lt_status upload(const float *h_x, const float *h_y, uint32_t n);
    lt_status move(float *dst, const float *src, uint64_t n, cudaMemcpyKind kind);
};

// use_net = false builds the frequency policy: the same decisions, scored by
// a moving average of visits instead of the network.
lt_status make_learned_policy(const lt_graph &g, int device, bool use_net, Policy **out);

}  // namespace lt
