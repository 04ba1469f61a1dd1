/* oracle/ref_shim/walk/SingleSource.h -- host stand-in for the initialiser
 * class app/ppr.cu names.  The reference's src/walk/SingleSource.h holds a
 * CUDA kernel launch that g++ cannot parse; the harness restates its
 * geometric walk length (SingleSource.h:11-18) itself.  Test infrastructure
 * only. */
#pragma once

template <typename Walker>
struct GPUSpecifiedNode {
    GPUSpecifiedNode(walkId, nodeId, float) {}
};
