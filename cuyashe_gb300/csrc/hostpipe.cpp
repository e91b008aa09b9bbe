// hostpipe.cpp -- entry points on host buffers whose copies overlap the kernels.
//
// The reference moves every operand to the device before a product and back
// after it, synchronously (Polynomial::update_device_data / update_host_data,
// src/polynomial.cpp:265-417; cudaDeviceSynchronize, src/common.h:223). Here a
// host-buffer call is cut into chunks that flow through six slots of device
// buffers: while chunks run their kernels, the next ones are copied in and the
// previous ones copied out, on a copy-in stream, three kernel streams (chunks are
// dealt round-robin so that neighbouring chunks' kernels overlap, as the lanes of
// the device-buffer calls do) and a copy-out stream. With page-locked host buffers the copies run on the copy engines
// alongside the kernels; pageable buffers give the same result, with copies
// that do not overlap.
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <map>
#include <mutex>

#include "host.h"

namespace cy {

constexpr int kPipeSlots = 6;  // chunks in flight (copy in, kernels, copy out)
constexpr int kRunStreams = 3;

// Per-device pipeline state, kept until process exit. Calls on one device take
// the pipeline in turn (the host blocks until a call's last copy is done).
struct HostPipe {
    std::mutex mu;
    cudaStream_t s_in = nullptr, s_run[kRunStreams] = {}, s_out = nullptr;
    struct Slot {
        uint64_t* d = nullptr;  // in0 | in1 | out, `words` each
        size_t words = 0;
        cudaEvent_t in_done = nullptr, run_done = nullptr, out_done = nullptr;
        bool used = false;
    } slot[kPipeSlots];
    cy_workspace ws[kRunStreams];  // one per kernel stream
};

static HostPipe& host_pipe(int dev) {
    static std::mutex mu;
    static std::map<int, HostPipe*> pipes;
    std::lock_guard<std::mutex> lock(mu);
    HostPipe*& p = pipes[dev];
    if (!p) p = new HostPipe();
    return *p;
}

static cy_status pipe_init(HostPipe& P, int dev) {
    if (P.s_in) return CY_OK;
    for (auto& w : P.ws) w.ws.device = dev;
    CY_CUDA(cudaStreamCreateWithFlags(&P.s_in, cudaStreamNonBlocking));
    for (auto& r : P.s_run) CY_CUDA(cudaStreamCreateWithFlags(&r, cudaStreamNonBlocking));
    CY_CUDA(cudaStreamCreateWithFlags(&P.s_out, cudaStreamNonBlocking));
    for (auto& s : P.slot) {
        CY_CUDA(cudaEventCreateWithFlags(&s.in_done, cudaEventDisableTiming));
        CY_CUDA(cudaEventCreateWithFlags(&s.run_done, cudaEventDisableTiming));
        CY_CUDA(cudaEventCreateWithFlags(&s.out_done, cudaEventDisableTiming));
    }
    return CY_OK;
}

// Slots are idle between calls (every call drains its streams before it returns).
static cy_status slot_reserve(HostPipe::Slot& s, size_t words) {
    if (s.words >= words) return CY_OK;
    if (s.d) cudaFree(s.d);
    s.d = nullptr;
    s.words = 0;
    CY_CUDA(cudaMalloc(&s.d, 3 * words * sizeof(uint64_t)));
    s.words = words;
    return CY_OK;
}

// Returns after the last result has reached h_out.
cy_status run_host_pipeline(size_t words, int batch, int chunk, const uint64_t* h_in0, const uint64_t* h_in1,
                            uint64_t* h_out, const ChunkOp& op) {
    if (batch <= 0) return CY_OK;
    int dev = 0;
    CY_CUDA(cudaGetDevice(&dev));
    HostPipe& P = host_pipe(dev);
    std::lock_guard<std::mutex> lock(P.mu);
    CY_TRY(pipe_init(P, dev));
    chunk = std::max(1, std::min(chunk, batch));
    // Chunk sizes: a quarter and a half chunk first, so that the kernels start
    // after a short copy, and a half and a quarter chunk last, so that the last
    // kernels and the last copy out are short; whole chunks between.
    std::vector<int> sizes;
    {
        const int q4 = std::max(1, chunk / 4), q2 = std::max(1, chunk / 2);
        int left = batch;
        if (left > 2 * chunk + q2 + q4) {
            sizes.push_back(q4);
            sizes.push_back(q2);
            left -= q4 + q2;
        }
        while (left > chunk + q2 + q4) {
            sizes.push_back(chunk);
            left -= chunk;
        }
        if (left > q2 + q4 && batch > 2 * chunk) {
            sizes.push_back(left - q2 - q4);
            sizes.push_back(q2);
            sizes.push_back(q4);
        } else {
            while (left > 0) {
                sizes.push_back(std::min(chunk, left));
                left -= sizes.back();
            }
        }
    }
    const int nchunks = (int)sizes.size();
    const int nslots = std::min(kPipeSlots, nchunks);
    const size_t cw = words * (size_t)chunk;
    for (int s = 0; s < nslots; s++) {
        CY_TRY(slot_reserve(P.slot[s], cw));
        P.slot[s].used = false;
    }
    cy_status st = CY_OK;
    cudaError_t e = cudaSuccess;
    int j0 = 0;
    for (int c = 0; c < nchunks && st == CY_OK && e == cudaSuccess; j0 += sizes[c], c++) {
        const int nj = sizes[c];
        HostPipe::Slot& S = P.slot[c % nslots];
        const size_t off = (size_t)j0 * words, bytes = (size_t)nj * words * sizeof(uint64_t);
        uint64_t *in0 = S.d, *in1 = S.d + S.words, *out = S.d + 2 * S.words;
        // copy in once the slot's previous chunk has consumed its inputs
        if (S.used) e = cudaStreamWaitEvent(P.s_in, S.run_done, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(in0, h_in0 + off, bytes, cudaMemcpyHostToDevice, P.s_in);
        if (e == cudaSuccess && h_in1)
            e = cudaMemcpyAsync(in1, h_in1 + off, bytes, cudaMemcpyHostToDevice, P.s_in);
        if (e == cudaSuccess) e = cudaEventRecord(S.in_done, P.s_in);
        // run once the inputs are in and the slot's previous output is out
        cudaStream_t run = P.s_run[c % kRunStreams];
        if (e == cudaSuccess) e = cudaStreamWaitEvent(run, S.in_done, 0);
        if (e == cudaSuccess && S.used) e = cudaStreamWaitEvent(run, S.out_done, 0);
        if (e != cudaSuccess) break;
        st = op(&P.ws[c % kRunStreams], in0, h_in1 ? in1 : nullptr, out, nj, run);
        if (st != CY_OK) break;
        e = cudaEventRecord(S.run_done, run);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(P.s_out, S.run_done, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(h_out + off, out, bytes, cudaMemcpyDeviceToHost, P.s_out);
        if (e == cudaSuccess) e = cudaEventRecord(S.out_done, P.s_out);
        S.used = true;
    }
    // drain every stream, whatever happened above
    const cudaError_t e1 = cudaStreamSynchronize(P.s_in);
    cudaError_t e2 = cudaSuccess;
    for (auto& r : P.s_run) {
        const cudaError_t e2b = cudaStreamSynchronize(r);
        if (e2 == cudaSuccess) e2 = e2b;
    }
    const cudaError_t e3 = cudaStreamSynchronize(P.s_out);
    if (st != CY_OK) return st;
    if (e != cudaSuccess) return cuda_error(e, "host pipeline");
    if (e1 != cudaSuccess) return cuda_error(e1, "host pipeline (copy in)");
    if (e2 != cudaSuccess) return cuda_error(e2, "host pipeline (kernels)");
    if (e3 != cudaSuccess) return cuda_error(e3, "host pipeline (copy out)");
    return CY_OK;
}

}  // namespace cy
