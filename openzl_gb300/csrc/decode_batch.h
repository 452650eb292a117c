// Batched decode of planned frames on the device, shared by the C entry
// points (capi.cpp) and the serving loop (server.cpp).
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/openzl_gb300.h"
#include "dec_exec.h"
#include "dec_plan.h"

namespace ozl {

inline ZL_Report reportOk(size_t v) { return ZL_Report{ ZL_ErrorCode_no_error, v }; }
inline ZL_Report reportFail(int code) { return ZL_Report{ ZL_ErrorCode(code), 0 }; }

// Grow-only device allocation with slack so that kernels may read whole
// aligned words around the ends of the streams they hold.
struct DevBuf {
    uint8_t* p = nullptr;
    size_t cap = 0;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    bool reserve(size_t bytes)
    {
        size_t const want = bytes + 256;
        if (want <= cap) return true;
        release();
        if (cudaMalloc(&p, want) != cudaSuccess) {
            p = nullptr;
            return false;
        }
        cap = want;
        return true;
    }
    uint8_t* data() const { return p ? p + 64 : nullptr; } // 64 bytes of slack in front
};

// Kernel attributes, set once per process.
cudaError_t prepareOnce();

// A planned decode of one or more frames, with its device resources.
//
// The frames are split into parts whose kernel chains share no launch: frames
// decoded through Huffman and the others. Part 0 runs on the caller's
// stream, the other parts on side streams forked from it and joined back by
// events, so that a CUDA graph captured from the caller's stream holds the
// parts as parallel branches (an FSE-heavy chain overlaps a Huffman-heavy
// one). All parts share the plan's arena and parameter block; each has its
// own descriptor pool and scratch.
struct DecodeBatch {
    static constexpr int kMaxParts = 2;
    struct Part {
        DeviceLayout layout;
        DevBuf pool, scratch;
        std::vector<char> mask;   // frames of this part
    };
    bool checkContent = true;
    bool checkCompressed = true;
    bool splitParts = true;
    DecodePlan plan;
    std::vector<Part> parts;
    DevBuf arena, params, status;
    std::vector<const uint8_t*> dFrames;
    std::vector<uint8_t*> dOuts;
    std::vector<size_t> sizes;
    long launches = 0;
    bool uploaded = false;   // descriptors and parameters of the plan are on the device
    cudaGraphExec_t graph = nullptr;
    cudaStream_t graphStream = nullptr;
    cudaStream_t side[kMaxParts] = {};
    cudaEvent_t fork = nullptr, join[kMaxParts] = {};
    std::string err;

    ~DecodeBatch()
    {
        dropGraph();
        for (int p = 0; p < kMaxParts; p++) {
            if (side[p]) cudaStreamDestroy(side[p]);
            if (join[p]) cudaEventDestroy(join[p]);
        }
        if (fork) cudaEventDestroy(fork);
    }
    void dropGraph()
    {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    const DeviceLayout& layoutOf(size_t p) const { return parts[p].layout; }
    size_t nbLaunches() const
    {
        size_t n = 0;
        for (const Part& p : parts) n += p.layout.launches.size();
        return n;
    }
    // launch i over all parts in order: (part, index within the part)
    bool locate(size_t i, size_t& part, size_t& li) const
    {
        for (size_t p = 0; p < parts.size(); p++) {
            if (i < parts[p].layout.launches.size()) {
                part = p;
                li = i;
                return true;
            }
            i -= parts[p].layout.launches.size();
        }
        return false;
    }

    ZL_Report makePlan(size_t n, const void* const* hF, const size_t* fs, const void* const* dF,
                       void* const* dO, const size_t* caps)
    {
        dropGraph();
        if (prepareOnce() != cudaSuccess) { err = "kernel attributes could not be set"; return reportFail(ZL_ErrorCode_GENERIC); }
        int rc = plan.build(n, reinterpret_cast<const uint8_t* const*>(hF), fs, caps, checkContent,
                            checkCompressed, err);
        if (rc) return reportFail(rc);
        dFrames.assign(reinterpret_cast<const uint8_t* const*>(dF), reinterpret_cast<const uint8_t* const*>(dF) + n);
        dOuts.assign(reinterpret_cast<uint8_t* const*>(dO), reinterpret_cast<uint8_t* const*>(dO) + n);
        sizes.resize(n);
        for (size_t i = 0; i < n; i++) sizes[i] = size_t(plan.frames[i].decodedSize);
        // parts: frames decoded through Huffman, then the others
        std::vector<char> huf(n, 0);
        for (const PlanNode& nd : plan.nodes)
            if (!nd.dead && nd.id == 50 && nd.frame >= 0) huf[size_t(nd.frame)] = 1;
        size_t nbHuf = 0;
        for (char h : huf) nbHuf += h;
        parts.clear();
        if (!splitParts || nbHuf == 0 || nbHuf == n) {
            parts.resize(1);
            parts[0].mask.assign(n, 1);
        } else {
            parts.resize(2);
            parts[0].mask.resize(n);
            parts[1].mask.resize(n);
            for (size_t i = 0; i < n; i++) {
                parts[0].mask[i] = char(!huf[i]);
                parts[1].mask[i] = huf[i];
            }
        }
        if (!arena.reserve(plan.arenaBytes) || !params.reserve(plan.params.size()) || !status.reserve(64)) {
            err = "device allocation failed";
            return reportFail(ZL_ErrorCode_allocation);
        }
        for (Part& p : parts) {
            // size pass, allocate, then the real layout
            const std::vector<char>* mask = parts.size() > 1 ? &p.mask : nullptr;
            rc = layoutPlan(plan, dFrames.data(), dOuts.data(), nullptr, nullptr, nullptr, nullptr, p.layout, err, mask);
            if (rc) return reportFail(rc);
            if (!p.pool.reserve(p.layout.pool.size()) || !p.scratch.reserve(p.layout.scratchBytes)) {
                err = "device allocation failed";
                return reportFail(ZL_ErrorCode_allocation);
            }
            rc = layoutPlan(plan, dFrames.data(), dOuts.data(), arena.data(), params.data(), p.scratch.data(),
                            p.pool.data(), p.layout, err, mask);
            if (rc) return reportFail(rc);
        }
        uploaded = false;
        launches = 0;
        return reportOk(size_t(plan.totalOut));
    }

    // Copies the plan's descriptors and parameters to the device, ordered on
    // the stream that runs the plan (the kernels read them).
    ZL_Report upload(cudaStream_t s)
    {
        if (uploaded) return reportOk(0);
        for (Part& p : parts)
            if (!p.layout.pool.empty()
                && cudaMemcpyAsync(p.pool.data(), p.layout.pool.data(), p.layout.pool.size(), cudaMemcpyHostToDevice, s)
                           != cudaSuccess) {
                err = "descriptor upload failed";
                return reportFail(ZL_ErrorCode_GENERIC);
            }
        if (!plan.params.empty()
            && cudaMemcpyAsync(params.data(), plan.params.data(), plan.params.size(), cudaMemcpyHostToDevice, s)
                       != cudaSuccess) {
            err = "parameter upload failed";
            return reportFail(ZL_ErrorCode_GENERIC);
        }
        uploaded = true;
        return reportOk(0);
    }

    ZL_Report enqueue(cudaStream_t s)
    {
        if (cudaMemsetAsync(status.data(), 0, 4, s) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
        uint32_t* const st = reinterpret_cast<uint32_t*>(status.data());
        size_t const np = parts.size();
        if (np > 1) {
            if (!fork && cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
            for (size_t p = 1; p < np; p++) {
                if (!side[p] && cudaStreamCreateWithFlags(&side[p], cudaStreamNonBlocking) != cudaSuccess)
                    return reportFail(ZL_ErrorCode_GENERIC);
                if (!join[p] && cudaEventCreateWithFlags(&join[p], cudaEventDisableTiming) != cudaSuccess)
                    return reportFail(ZL_ErrorCode_GENERIC);
            }
            cudaEventRecord(fork, s);
            for (size_t p = 1; p < np; p++) cudaStreamWaitEvent(side[p], fork, 0);
        }
        long total = 0;
        for (size_t p = 0; p < np; p++) {
            cudaStream_t const ps = p == 0 ? s : side[p];
            long n = runLaunches(parts[p].layout, parts[p].pool.data(), parts[p].scratch.data(), st, ps);
            if (n < 0) {
                err = std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError());
                return reportFail(ZL_ErrorCode_GENERIC);
            }
            total += n;
        }
        for (size_t p = 1; p < np; p++) {
            cudaEventRecord(join[p], side[p]);
            cudaStreamWaitEvent(s, join[p], 0);
        }
        launches = total;
        return reportOk(0);
    }

    ZL_Report run(cudaStream_t s, bool useGraph)
    {
        ZL_Report const u = upload(s);
        if (ZL_isError(u)) return u;
        if (!useGraph) return enqueue(s);
        if (s == nullptr) {
            err = "CUDA graph capture needs a non-default stream";
            return reportFail(ZL_ErrorCode_parameter_invalid);
        }
        if (!graph || graphStream != s) {
            dropGraph();
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                err = "stream capture failed";
                return reportFail(ZL_ErrorCode_GENERIC);
            }
            ZL_Report r = enqueue(s);
            cudaError_t e = cudaStreamEndCapture(s, &g);
            if (ZL_isError(r)) { if (g) cudaGraphDestroy(g); return r; }
            if (e != cudaSuccess) { err = "stream capture failed"; return reportFail(ZL_ErrorCode_GENERIC); }
            e = cudaGraphInstantiate(&graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { graph = nullptr; err = "graph instantiation failed"; return reportFail(ZL_ErrorCode_GENERIC); }
            graphStream = s;
        }
        if (cudaGraphLaunch(graph, s) != cudaSuccess) { err = "graph launch failed"; return reportFail(ZL_ErrorCode_GENERIC); }
        return reportOk(0);
    }

    // Times every candidate launch shape of the tunable launches (one launch
    // at a time, CUDA events on `s`, best of `reps`) after one full run that
    // produces every launch's inputs, keeps the fastest per launch and drops
    // the captured graph. Returns the number of launches tuned.
    ZL_Report autotune(cudaStream_t s, int reps)
    {
        ZL_Report r = upload(s);
        if (ZL_isError(r)) return r;
        r = enqueue(s);
        if (ZL_isError(r)) return r;
        if (cudaStreamSynchronize(s) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
        cudaEvent_t a = nullptr, b = nullptr;
        if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
        size_t tuned = 0;
        for (Part& part : parts) {
            for (size_t li = 0; li < part.layout.launches.size(); li++) {
                uint32_t cand[8];
                uint32_t const nc = tuneCandidates(part.layout.launches[li], cand, 8);
                if (nc < 2) continue;
                float best = 1e30f;
                uint32_t bestC = 0;
                for (uint32_t k = 0; k < nc; k++) {
                    part.layout.launches[li].tune = cand[k];
                    float t = 1e30f;
                    for (int rep = 0; rep < reps; rep++) {
                        cudaEventRecord(a, s);
                        if (runOneLaunch(part.layout, li, part.pool.data(), part.scratch.data(),
                                         reinterpret_cast<uint32_t*>(status.data()), s) < 0)
                            break;
                        cudaEventRecord(b, s);
                        cudaEventSynchronize(b);
                        float ms = 0;
                        cudaEventElapsedTime(&ms, a, b);
                        t = ms < t ? ms : t;
                    }
                    if (t < best) { best = t; bestC = cand[k]; }
                }
                part.layout.launches[li].tune = bestC;
                tuned++;
            }
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        dropGraph();
        if (cudaStreamSynchronize(s) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
        return reportOk(tuned);
    }

    ZL_Report check(cudaStream_t s)
    {
        uint32_t st = 0;
        if (cudaMemcpyAsync(&st, status.data(), 4, cudaMemcpyDeviceToHost, s) != cudaSuccess
            || cudaStreamSynchronize(s) != cudaSuccess) {
            err = std::string("device error: ") + cudaGetErrorString(cudaGetLastError());
            return reportFail(ZL_ErrorCode_GENERIC);
        }
        if (st) {
            err = st == 13 ? "compressed checksum mismatch"
                           : st == 14 ? "content checksum mismatch" : st == 80 ? "device wait timed out" : "corruption";
            return reportFail(int(st));
        }
        return reportOk(size_t(plan.totalOut));
    }
};

} // namespace ozl
