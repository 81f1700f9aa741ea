// Conditional WHILE nodes in stream capture (shared by the solvers).
#pragma once
#include <cuda_runtime.h>

namespace f2d {

// add a WHILE node at the current capture position of `st` and capture its
// body with `rec(stream)` on `sb`
template <typename R>
inline int add_while(cudaStream_t st, cudaStream_t sb, cudaGraphConditionalHandle* cond,
                     unsigned dflt, R rec)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
    if (e != cudaSuccess) return (int)e;
    if (!*cond) {
        e = cudaGraphConditionalHandleCreate(cond, graph, dflt, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return (int)e;
    }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = *cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp);
    if (e != cudaSuccess) return (int)e;
    e = cudaStreamBeginCaptureToGraph(sb, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return (int)e;
    int r = rec(sb);
    cudaGraph_t out;
    e = cudaStreamEndCapture(sb, &out);
    if (r) return r;
    if (e != cudaSuccess) return (int)e;
    return (int)cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                                    cudaStreamSetCaptureDependencies);
}

}  // namespace f2d
