/* oracle/ref_shim/walk/NodeSampler.h -- host stand-in for the initialiser
 * class app/pagerank.cu and app/genericwalk.cu name.  The reference's
 * src/walk/NodeSampler.h holds a CUDA kernel launch that g++ cannot parse;
 * the harness restates its uniform start (NodeSampler.h:10-13) itself.  Test
 * infrastructure only. */
#pragma once

template <typename Walker>
struct GPUNodeSampler {
    GPUNodeSampler(walkId, nodeId, nodeId) {}
};
