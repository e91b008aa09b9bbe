// graph.cpp -- a fixed batch of products or HE multiplies captured once as a
// CUDA graph and replayed.
//
// Every entry point of the multiply path only launches kernels on the caller's
// stream once its workspace has grown (no allocation, no host synchronisation),
// so a call can be recorded with stream capture. The graph owns a workspace
// that is grown by one untimed call before capture; each replay then costs one
// graph launch instead of one launch per kernel and chunk. The reference
// synchronises the device after every operation (src/common.h:223,
// src/cuda_functions.cu:738).
#include <cuda_runtime.h>

#include <functional>
#include <memory>

#include "host.h"

struct cy_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cy_workspace ws;
    ~cy_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

namespace cy {

// Runs `op` once to grow the workspace, then records it on a private stream.
static cy_status capture(const std::function<cy_status(cy_workspace*, cudaStream_t)>& op, cy_graph** out) {
    std::unique_ptr<cy_graph> g(new cy_graph());
    CY_CUDA(cudaGetDevice(&g->ws.ws.device));
    cudaStream_t st = nullptr;
    CY_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cy_status s = op(&g->ws, st);
    if (s == CY_OK) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            s = cuda_error(e, "cudaStreamBeginCapture");
        } else {
            s = op(&g->ws, st);
            cudaGraph_t graph = nullptr;
            e = cudaStreamEndCapture(st, &graph);
            if (s == CY_OK && e != cudaSuccess) s = cuda_error(e, "cudaStreamEndCapture");
            g->graph = graph;
            if (s == CY_OK) {
                e = cudaGraphInstantiate(&g->exec, graph, 0);
                if (e != cudaSuccess) s = cuda_error(e, "cudaGraphInstantiate");
            }
        }
    }
    cudaStreamDestroy(st);
    if (s != CY_OK) return s;
    *out = g.release();
    return CY_OK;
}

}  // namespace cy

using namespace cy;

extern "C" {

cy_status cy_polymul_graph_create(cy_ring* ring, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_c, int batch,
                                  cy_graph** out) {
    if (!ring || !out || batch < 1 || !d_a || !d_b || !d_c) return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    return capture([=](cy_workspace* ws, cudaStream_t st) { return cy_polymul_ws(ring, ws, d_a, d_b, d_c, batch, st); },
                   out);
}

cy_status cy_yashe_mul_graph_create(cy_yashe* y, const uint64_t* d_c1, const uint64_t* d_c2, uint64_t* d_out,
                                    int batch, int relin, cy_graph** out) {
    if (!y || !out || batch < 1 || !d_c1 || !d_c2 || !d_out) return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    return capture(
        [=](cy_workspace* ws, cudaStream_t st) { return cy_yashe_mul_ws(y, ws, d_c1, d_c2, d_out, batch, relin, st); },
        out);
}

cy_status cy_mixed_plan_graph_create(cy_mixed_plan* plan, cy_graph** out) {
    if (!plan || !out) return set_error(CY_ERR_INVALID_ARGUMENT, "bad argument");
    return capture([=](cy_workspace*, cudaStream_t st) { return cy_mixed_plan_launch(plan, st); }, out);
}

cy_status cy_graph_launch(cy_graph* g, cy_stream_t stream) {
    if (!g || !g->exec) return set_error(CY_ERR_INVALID_ARGUMENT, "graph is NULL");
    CY_CUDA(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    return CY_OK;
}

cy_status cy_graph_destroy(cy_graph* g) {
    delete g;
    return CY_OK;
}

}  // extern "C"
