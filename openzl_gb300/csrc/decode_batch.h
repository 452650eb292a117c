// Batched decode of planned frames on the device, shared by the C entry
// points (capi.cpp) and the serving loop (server.cpp).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "../../include/openzl_gb300.h"
#include "dec_exec.h"
#include "dec_plan.h"
#include "device_scope.h"

namespace ozl {

inline ZL_Report reportOk(size_t v) { return ZL_Report{ ZL_ErrorCode_no_error, v }; }
// Decoded size of a single-output frame (whole header parsed; several
// outputs refused), for the library's own decode calls (capi.cpp).
ZL_Report singleOutputSize(const void* src, size_t size);
inline ZL_Report reportFail(int code) { return ZL_Report{ ZL_ErrorCode(code), 0 }; }

// Grow-only device allocation with slack so that kernels may read whole
// aligned words around the ends of the streams they hold.
struct DevBuf {
    uint8_t* p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), cap(o.cap)
    {
        o.p = nullptr;
        o.cap = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            cap = o.cap;
            o.p = nullptr;
            o.cap = 0;
        }
        return *this;
    }
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
// parts as parallel branches: an FSE-heavy chain overlaps a Huffman-heavy
// one, and each kind splits into runs of contiguous frames so that one run's
// bandwidth-bound levels (numeric pipeline, checksums) overlap another run's
// latency-bound entropy decoding. All parts share the plan's arena and
// parameter block; each has its own descriptor pool and scratch.
struct DecodeBatch {
    static constexpr int kMaxParts = 17; // the critical part plus 8 runs of each of two kinds
    struct Part {
        DeviceLayout layout;
        DevBuf pool, scratch;
        std::vector<char> mask;   // frames of this part
        bool critical = false;    // frames with a long FSE stream: highest stream priority
        int run = 0;              // index of this run within its kind
    };
    bool checkContent = true;
    bool checkCompressed = true;
    bool splitParts = true;
    int partsPerKind = 0;     // runs per kind (OZL_DParam_partsPerKind); 0 = by batch size
    int fseKernel = 0;        // OZL_DParam_fseKernel: 0 default shapes, 1 a lane per stream, 2 a lane per state
    int64_t criticalSymbols = -1; // OZL_DParam_criticalSymbols: 0 = no critical part, -1 = by batch size
    // Batches decoding at least this many bytes split by default into a
    // critical part (FSE streams of 16,000 symbols or more) and two runs per
    // kind; smaller ones into the Huffman frames and the others.
    static constexpr uint64_t kSplitBytes = 512ull << 20;
    static constexpr uint32_t kCriticalDefault = 16000;
    int schedule = 0;             // OZL_DParam_schedule: priority policy of the branches
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
    std::map<uint64_t, std::pair<cudaStream_t, int>> slots; // launch-slot streams and their priorities
    std::vector<cudaEvent_t> events;                         // dependency events of a run
    std::string err;

    // Host-buffer runs (ozl_gpu_batch_run_host): the frames split into
    // rounds of contiguous frames. Each round's frames go up on one copy
    // stream, the round decodes on its own stream as soon as they are in
    // (rounds share the SMs), and its outputs go down on a second copy stream
    // as soon as it is done, so both copy directions overlap the decode.
    unsigned planThreads = 0; // host threads of the plan build (0: the machine's, at most 8)
    int hostRounds = 16;     // OZL_DParam_hostRounds
    int hostDepth = 6;       // OZL_DParam_hostDepth: rounds decoding at once (0 = all)
    struct HostPipe {
        static constexpr int kRounds = 16;
        std::vector<Part> rounds;
        std::vector<size_t> inOff, outOff; // round boundaries in the input / output images
        bool ready = false, uploaded = false;
        cudaStream_t sIn = nullptr, sOut = nullptr, rs[kRounds] = {};
        cudaEvent_t start = nullptr, inEv[kRounds] = {}, decEv[kRounds] = {}, outDone = nullptr;
        cudaGraphExec_t graph = nullptr;
        const void* gIn = nullptr;
        void* gOut = nullptr;
        size_t gInBytes = 0, gOutBytes = 0;
        cudaStream_t gStream = nullptr;
        void dropGraph()
        {
            if (graph) cudaGraphExecDestroy(graph);
            graph = nullptr;
        }
        void reset() // keeps the rounds' device buffers for the next plan
        {
            dropGraph();
            ready = uploaded = false;
        }
        ~HostPipe()
        {
            dropGraph();
            if (sIn) cudaStreamDestroy(sIn);
            if (sOut) cudaStreamDestroy(sOut);
            for (int r = 0; r < kRounds; r++) {
                if (rs[r]) cudaStreamDestroy(rs[r]);
                if (inEv[r]) cudaEventDestroy(inEv[r]);
                if (decEv[r]) cudaEventDestroy(decEv[r]);
            }
            if (start) cudaEventDestroy(start);
            if (outDone) cudaEventDestroy(outDone);
        }
    } host;

    ~DecodeBatch()
    {
        if (lastRun) cudaEventDestroy(lastRun);
        dropGraph();
        for (auto& kv : slots) cudaStreamDestroy(kv.second.first);
        for (cudaEvent_t e : events) cudaEventDestroy(e);
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
        host.reset();
        if (prepareOnce() != cudaSuccess) { err = "kernel attributes could not be set"; return reportFail(ZL_ErrorCode_GENERIC); }
        unsigned const hw = std::thread::hardware_concurrency();
        unsigned const threads = planThreads ? planThreads : std::min(8u, hw ? hw : 1u);
        int rc = plan.buildParallel(n, reinterpret_cast<const uint8_t* const*>(hF), fs, caps, checkContent,
                                    checkCompressed, err, threads);
        if (rc) return reportFail(rc);
        dFrames.assign(reinterpret_cast<const uint8_t* const*>(dF), reinterpret_cast<const uint8_t* const*>(dF) + n);
        dOuts.assign(reinterpret_cast<uint8_t* const*>(dO), reinterpret_cast<uint8_t* const*>(dO) + n);
        sizes.resize(n);
        for (size_t i = 0; i < n; i++) sizes[i] = size_t(plan.frames[i].decodedSize);
        // parts: frames holding an FSE stream of at least criticalSymbols
        // symbols (decoded serially by one lane each, so they are the batch's
        // longest chains), the frames decoded through Huffman (transform 50),
        // and the others. Each kind splits into runs of contiguous frames of
        // about equal decoded bytes.
        bool const big = plan.totalOut >= kSplitBytes;
        int const runs = partsPerKind ? partsPerKind : big ? 2 : 1;
        uint64_t const critical = criticalSymbols >= 0 ? uint64_t(criticalSymbols) : big ? kCriticalDefault : 0;
        std::vector<char> kindOf(n, 0);
        for (const PlanNode& nd : plan.nodes)
            if (!nd.dead && nd.id == 50 && nd.frame >= 0) kindOf[size_t(nd.frame)] = 1;
        if (critical)
            for (const PlanNode& nd : plan.nodes)
                if (!nd.dead && nd.id == 49 && nd.frame >= 0 && nd.out >= 0
                    && plan.streams[size_t(nd.out)].n >= critical)
                    kindOf[size_t(nd.frame)] = 2;
        // the parts' device buffers outlive the plan: a new plan reuses them
        // (no allocation, and so no device-wide synchronization, per batch)
        struct Spec {
            std::vector<char> mask;
            bool critical;
            int run;
        };
        std::vector<Spec> specs;
        if (splitParts) {
            for (char kind : { char(2), char(1), char(0) }) {
                std::vector<size_t> fr;
                uint64_t total = 0;
                for (size_t i = 0; i < n; i++)
                    if (kindOf[i] == kind) {
                        fr.push_back(i);
                        total += sizes[i];
                    }
                if (fr.empty()) continue;
                size_t const g = kind == 2 ? 1 : std::min<size_t>(size_t(runs), fr.size());
                size_t const first = specs.size();
                for (size_t k = 0; k < g; k++) specs.push_back(Spec{ std::vector<char>(n, 0), kind == 2, int(k) });
                uint64_t acc = 0;
                size_t k = 0;
                for (size_t i : fr) {
                    while (k + 1 < g && acc >= total * (k + 1) / g) k++;
                    specs[first + k].mask[i] = 1;
                    acc += sizes[i];
                }
            }
        }
        if (specs.empty()) specs.push_back(Spec{ std::vector<char>(n, 1), false, 0 });
        if (specs.size() > size_t(kMaxParts)) {
            err = "too many parts";
            return reportFail(ZL_ErrorCode_parameter_invalid);
        }
        parts.resize(specs.size());
        for (size_t p = 0; p < specs.size(); p++) {
            parts[p].mask = std::move(specs[p].mask);
            parts[p].critical = specs[p].critical;
            parts[p].run = specs[p].run;
            parts[p].layout = DeviceLayout();
        }
        if (!arena.reserve(plan.arenaBytes) || !params.reserve(plan.params.size()) || !status.reserve(64)) {
            err = "device allocation failed";
            return reportFail(ZL_ErrorCode_allocation);
        }
        // Each part's layout: one pass into the part's buffers when they are
        // large enough (they outlive plans), else a size pass, a larger
        // allocation and the real pass. Parts only read the plan, so large
        // batches lay them out on parallel host threads.
        std::vector<int> prc(parts.size(), 0);
        std::vector<std::string> perr(parts.size());
        auto layoutPart = [&](size_t k) {
            Part& p = parts[k];
            const std::vector<char>* mask = parts.size() > 1 ? &p.mask : nullptr;
            if (p.pool.data() && p.scratch.data()) {
                prc[k] = layoutPlan(plan, dFrames.data(), dOuts.data(), arena.data(), params.data(), p.scratch.data(),
                                    p.pool.data(), p.layout, perr[k], mask);
                if (prc[k] || (p.layout.pool.size() + 256 <= p.pool.cap && p.layout.scratchBytes + 256 <= p.scratch.cap))
                    return;
            }
            prc[k] = layoutPlan(plan, dFrames.data(), dOuts.data(), nullptr, nullptr, nullptr, nullptr, p.layout,
                                perr[k], mask);
            if (prc[k]) return;
            if (!p.pool.reserve(p.layout.pool.size()) || !p.scratch.reserve(p.layout.scratchBytes)) {
                prc[k] = ZL_ErrorCode_allocation;
                perr[k] = "device allocation failed";
                return;
            }
            prc[k] = layoutPlan(plan, dFrames.data(), dOuts.data(), arena.data(), params.data(), p.scratch.data(),
                                p.pool.data(), p.layout, perr[k], mask);
        };
        if (parts.size() > 1 && n >= 64) {
            std::vector<std::thread> th;
            for (size_t k = 1; k < parts.size(); k++) th.emplace_back(layoutPart, k);
            layoutPart(0);
            for (std::thread& t : th) t.join();
        } else {
            for (size_t k = 0; k < parts.size(); k++) layoutPart(k);
        }
        for (size_t k = 0; k < parts.size(); k++)
            if (prc[k]) {
                err = perr[k];
                return reportFail(prc[k]);
            }
        for (Part& p : parts) applyFseKernel(p.layout);
        uploaded = false;
        launches = 0;
        return reportOk(size_t(plan.totalOut));
    }

    // Copies the plan's descriptors and parameters to the device, ordered on
    // the stream that runs the plan (the kernels read them).
    // The last run's end on its stream: a new plan's uploads (descriptors,
    // parameters) wait for it, since the buffers are reused across plans and
    // that run may be on another stream.
    cudaEvent_t lastRun = nullptr;
    void markRun(cudaStream_t s)
    {
        if (lastRun || cudaEventCreateWithFlags(&lastRun, cudaEventDisableTiming) == cudaSuccess) cudaEventRecord(lastRun, s);
    }
    void afterLastRun(cudaStream_t s)
    {
        if (lastRun) cudaStreamWaitEvent(s, lastRun, 0);
    }

    ZL_Report upload(cudaStream_t s)
    {
        if (uploaded) return reportOk(0);
        afterLastRun(s);
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

    // Stream of one launch slot: (part, position within its level, priority
    // class). Kept across runs; recreated when its priority changes.
    cudaStream_t slotStream(size_t part, size_t slot, int cls, int prio)
    {
        uint64_t const key = (uint64_t(part) << 24) | (uint64_t(slot) << 4) | uint64_t(cls);
        auto it = slots.find(key);
        if (it != slots.end() && it->second.second == prio) return it->second.first;
        if (it != slots.end()) {
            cudaStreamDestroy(it->second.first);
            slots.erase(it);
        }
        cudaStream_t x = nullptr;
        if (cudaStreamCreateWithPriority(&x, cudaStreamNonBlocking, prio) != cudaSuccess) return nullptr;
        slots.emplace(key, std::make_pair(x, prio));
        return x;
    }
    // the k-th event of this run (created once, reused by later runs)
    cudaEvent_t nextEvent(size_t& k)
    {
        if (k == events.size()) {
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
            events.push_back(e);
        }
        return events[k++];
    }

    // Enqueues the plan on `s` as a DAG: each part (branch) runs its
    // dependency levels in order, and the launches of one level, which do not
    // depend on one another, on streams of their own. Stream priorities
    // order the block scheduler's work. Schedule 0: a branch's launches share
    // its rank: the critical part (the longest chains) first, then each
    // kind's runs in order, so that a run's element-wise work shares the SMs
    // with the next run's entropy decoding. Schedule 1: every element-wise
    // launch (short, memory-bound) ahead of all entropy decoding, which keeps
    // the branch ranks. `marks` (timeline runs): a timing event before and
    // after every launch, in part order, on its stream.
    ZL_Report enqueue(cudaStream_t s, const std::vector<cudaEvent_t>* marks = nullptr)
    {
        if (cudaMemsetAsync(status.data(), 0, 4, s) != cudaSuccess) {
            err = "status reset failed";
            return reportFail(ZL_ErrorCode_GENERIC);
        }
        uint32_t* const st = reinterpret_cast<uint32_t*>(status.data());
        if (parts.size() == 1 && !marks) { // one branch: its launches in order on `s`
            long const n = runLaunches(parts[0].layout, parts[0].pool.data(), parts[0].scratch.data(), st, s);
            if (n < 0) {
                err = std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError());
                return reportFail(ZL_ErrorCode_GENERIC);
            }
            launches = n;
            return reportOk(0);
        }
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = greatest = 0;
        bool anyCritical = false;
        for (const Part& p : parts) anyCritical = anyCritical || p.critical;
        auto prioOf = [&](const Part& p, int kind) {
            int const branch = p.critical ? 0 : p.run + (anyCritical ? 1 : 0);
            bool const entropy = kind == KIND_FSE || kind == KIND_HUF || kind == KIND_HUF16;
            int const rank = schedule == 1 ? (entropy ? 1 + branch : 0) : branch;
            return std::min(least, greatest + rank); // greatest is the numerically smallest
        };
        size_t ev = 0;
        cudaEvent_t const start = nextEvent(ev);
        if (!start || cudaEventRecord(start, s) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
        long total = 0;
        size_t mark = 0;
        std::vector<cudaEvent_t> ends;
        for (size_t p = 0; p < parts.size(); p++) {
            const DeviceLayout& L = parts[p].layout;
            cudaEvent_t ready = start; // everything the next level waits for
            for (size_t a = 0; a < L.launches.size();) {
                size_t b = a;
                while (b < L.launches.size() && L.launches[b].level == L.launches[a].level) b++;
                std::vector<cudaStream_t> used;
                std::vector<cudaEvent_t> done;
                for (size_t li = a; li < b; li++, mark += 2) {
                    int const cls = (L.launches[li].kind == KIND_FSE || L.launches[li].kind == KIND_HUF
                                     || L.launches[li].kind == KIND_HUF16) ? 1 : 0;
                    cudaStream_t const x = slotStream(p, li - a, cls, prioOf(parts[p], L.launches[li].kind));
                    cudaEvent_t const e = nextEvent(ev);
                    if (!x || !e || cudaStreamWaitEvent(x, ready, 0) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
                    if (marks) cudaEventRecord((*marks)[mark], x);
                    long const k = runOneLaunch(L, li, parts[p].pool.data(), parts[p].scratch.data(), st, x);
                    if (marks) cudaEventRecord((*marks)[mark + 1], x);
                    if (k < 0) {
                        err = std::string("kernel launch failed: ") + cudaGetErrorString(cudaGetLastError());
                        return reportFail(ZL_ErrorCode_GENERIC);
                    }
                    total += k;
                    if (cudaEventRecord(e, x) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
                    used.push_back(x);
                    done.push_back(e);
                }
                if (done.size() == 1) {
                    ready = done[0];
                } else {
                    // join the level on its first stream
                    for (size_t k = 1; k < done.size(); k++) cudaStreamWaitEvent(used[0], done[k], 0);
                    cudaEvent_t const j = nextEvent(ev);
                    if (!j || cudaEventRecord(j, used[0]) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
                    ready = j;
                }
                a = b;
            }
            ends.push_back(ready);
        }
        for (cudaEvent_t e : ends)
            if (cudaStreamWaitEvent(s, e, 0) != cudaSuccess) return reportFail(ZL_ErrorCode_GENERIC);
        launches = total;
        return reportOk(0);
    }

    // One run without a graph, branches as in run(), with a timing event
    // around every launch. Row i of `rows` (5 floats, launches in part
    // order): part, kind, level, the ms from the run's start at which the
    // launch's stream reached it, and the ms at which it ended. A launch may
    // wait for SMs after its stream reaches it, so the gap between the two
    // bounds its time from above. Synchronizes `s`.
    ZL_Report timeline(cudaStream_t s, float* rows, size_t capacity)
    {
        ZL_Report const u = upload(s);
        if (ZL_isError(u)) return u;
        size_t const n = nbLaunches();
        std::vector<cudaEvent_t> marks(2 * n, nullptr);
        cudaEvent_t start = nullptr;
        bool ok = cudaEventCreate(&start) == cudaSuccess;
        for (auto& e : marks) ok = ok && cudaEventCreate(&e) == cudaSuccess;
        ZL_Report r = reportOk(0);
        if (ok) {
            cudaEventRecord(start, s);
            r = enqueue(s, &marks);
            ok = !ZL_isError(r) && cudaStreamSynchronize(s) == cudaSuccess;
        }
        size_t i = 0;
        for (size_t p = 0; ok && p < parts.size(); p++)
            for (size_t li = 0; li < parts[p].layout.launches.size(); li++, i++) {
                if (i >= capacity) continue;
                float a = 0, b = 0;
                cudaEventElapsedTime(&a, start, marks[2 * i]);
                cudaEventElapsedTime(&b, start, marks[2 * i + 1]);
                const Launch& l = parts[p].layout.launches[li];
                float* row = rows + 5 * i;
                row[0] = float(p);
                row[1] = float(l.kind);
                row[2] = float(l.level);
                row[3] = a;
                row[4] = b;
            }
        for (auto& e : marks)
            if (e) cudaEventDestroy(e);
        if (start) cudaEventDestroy(start);
        if (ZL_isError(r)) return r;
        if (!ok) {
            err = "timeline run failed";
            return reportFail(ZL_ErrorCode_GENERIC);
        }
        return reportOk(n);
    }

    ZL_Report run(cudaStream_t s, bool useGraph)
    {
        ZL_Report const u = upload(s);
        if (ZL_isError(u)) return u;
        if (!useGraph) {
            ZL_Report const r = enqueue(s);
            if (!ZL_isError(r)) markRun(s);
            return r;
        }
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
            // per-node priorities: the captured branches keep their streams' priorities
            e = cudaGraphInstantiateWithFlags(&graph, g, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { graph = nullptr; err = "graph instantiation failed"; return reportFail(ZL_ErrorCode_GENERIC); }
            graphStream = s;
        }
        if (cudaGraphLaunch(graph, s) != cudaSuccess) { err = "graph launch failed"; return reportFail(ZL_ErrorCode_GENERIC); }
        markRun(s);
        return reportOk(0);
    }

    // One host-buffer run without a graph, with timing events: row r of
    // `rows` (3 floats) holds the ms from the run's start at which round r's
    // frames were in, its decode ended and its outputs were out. Returns the
    // number of rounds (0 when the frames are not laid out in order for
    // rounds). Synchronizes `s`.
    ZL_Report hostTimeline(const void* hIn, size_t inBytes, void* hOut, size_t outBytes, cudaStream_t s, float* rows,
                           size_t capacity)
    {
        if (!buildRounds(inBytes, outBytes)) return reportOk(0);
        ZL_Report u = upload(s);
        if (ZL_isError(u)) return u;
        if (!host.uploaded) {
            afterLastRun(s);
            for (Part& p : host.rounds)
                if (!p.layout.pool.empty())
                    cudaMemcpyAsync(p.pool.data(), p.layout.pool.data(), p.layout.pool.size(), cudaMemcpyHostToDevice, s);
            host.uploaded = true;
        }
        size_t const nr = host.rounds.size();
        std::vector<cudaEvent_t> marks(1 + 3 * nr, nullptr);
        bool ok = true;
        for (auto& e : marks) ok = ok && cudaEventCreate(&e) == cudaSuccess;
        ZL_Report r = reportOk(nr);
        if (ok) {
            r = enqueueHost(hIn, hOut, s, &marks);
            if (!ZL_isError(r)) markRun(s);
            ok = !ZL_isError(r) && cudaStreamSynchronize(s) == cudaSuccess;
        }
        for (size_t k = 0; ok && k < 3 * nr && k < 3 * capacity; k++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, marks[0], marks[1 + k]);
            rows[k] = ms;
        }
        for (auto& e : marks)
            if (e) cudaEventDestroy(e);
        if (ZL_isError(r)) return r;
        if (!ok) {
            err = "host timeline run failed";
            return reportFail(ZL_ErrorCode_GENERIC);
        }
        ZL_Report const c = check(s);
        if (ZL_isError(c)) return c;
        return reportOk(nr);
    }

    // OZL_DParam_fseKernel: the FSE launches' kernel until the autotuner runs
    void applyFseKernel(DeviceLayout& layout) const
    {
        if (!fseKernel) return;
        for (Launch& l : layout.launches)
            if (l.kind == KIND_FSE) l.tune = fseKernel == 2 ? (kTuneFseLanePerState | 8u) : (l.param0 <= 8 ? 32u : 6u);
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
                uint32_t cand[16];
                uint32_t const nc = tuneCandidates(part.layout.launches[li], cand, 16);
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

    // Rounds for host-buffer runs: frames must be laid out in order in both
    // images (increasing device addresses inside [0, inBytes) and
    // [0, outBytes)); otherwise returns false and the caller runs the copies
    // and the decode one after another.
    bool buildRounds(size_t inBytes, size_t outBytes)
    {
        size_t const n = dFrames.size();
        if (n < 2) return false;
        for (size_t i = 0; i < n; i++) {
            size_t const fi = size_t(dFrames[i] - dFrames[0]), oi = size_t(dOuts[i] - dOuts[0]);
            if (dFrames[i] < dFrames[0] || dOuts[i] < dOuts[0] || fi >= inBytes || oi + sizes[i] > outBytes) return false;
            if (i && (dFrames[i] < dFrames[i - 1] || dOuts[i] < dOuts[i - 1] + sizes[i - 1])) return false;
        }
        if (host.ready) return true;
        int const K = int(std::min<size_t>(size_t(hostRounds), n));
        uint64_t const target = (plan.totalOut + K - 1) / K;
        std::vector<size_t> first{ 0 };
        uint64_t acc = 0;
        for (size_t i = 0; i + 1 < n && int(first.size()) < K; i++) {
            acc += sizes[i];
            if (acc >= target * first.size()) first.push_back(i + 1);
        }
        first.push_back(n);
        size_t const nr = first.size() - 1;
        host.rounds.resize(nr);
        host.inOff.assign(nr + 1, 0);
        host.outOff.assign(nr + 1, 0);
        for (size_t r = 0; r < nr; r++) {
            Part& p = host.rounds[r];
            p.mask.assign(n, 0);
            for (size_t i = first[r]; i < first[r + 1]; i++) p.mask[i] = 1;
            bool fits = false;
            if (p.pool.data() && p.scratch.data()) { // one pass into buffers kept from an earlier plan
                if (layoutPlan(plan, dFrames.data(), dOuts.data(), arena.data(), params.data(), p.scratch.data(),
                               p.pool.data(), p.layout, err, &p.mask))
                    return false;
                fits = p.layout.pool.size() + 256 <= p.pool.cap && p.layout.scratchBytes + 256 <= p.scratch.cap;
            }
            if (!fits) {
                int rc = layoutPlan(plan, dFrames.data(), dOuts.data(), nullptr, nullptr, nullptr, nullptr, p.layout,
                                    err, &p.mask);
                if (rc) return false;
                if (!p.pool.reserve(p.layout.pool.size()) || !p.scratch.reserve(p.layout.scratchBytes)) return false;
                rc = layoutPlan(plan, dFrames.data(), dOuts.data(), arena.data(), params.data(), p.scratch.data(),
                                p.pool.data(), p.layout, err, &p.mask);
                if (rc) return false;
            }
            applyFseKernel(p.layout);
            host.inOff[r] = size_t(dFrames[first[r]] - dFrames[0]);
            host.outOff[r] = size_t(dOuts[first[r]] - dOuts[0]);
        }
        host.inOff[nr] = inBytes;
        host.outOff[nr] = outBytes;
        // earlier rounds decode at higher stream priority, so they finish
        // first and their outputs start down while later rounds fill the SMs
        int least = 0, greatest = 0;
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = greatest = 0;
        auto mkStream = [](cudaStream_t& x, int prio) {
            return x || cudaStreamCreateWithPriority(&x, cudaStreamNonBlocking, prio) == cudaSuccess;
        };
        auto mkEvent = [](cudaEvent_t& x) { return x || cudaEventCreateWithFlags(&x, cudaEventDisableTiming) == cudaSuccess; };
        bool ok = mkStream(host.sIn, greatest) && mkStream(host.sOut, greatest) && mkEvent(host.start)
                  && mkEvent(host.outDone);
        for (size_t r = 0; r < nr && ok; r++) {
            int const prio = nr > 1 ? greatest + int((int64_t(least) - greatest) * int64_t(r) / int64_t(nr - 1)) : greatest;
            ok = mkStream(host.rs[r], prio) && mkEvent(host.inEv[r]) && mkEvent(host.decEv[r]);
        }
        if (!ok) return false;
        host.ready = true;
        host.uploaded = false;
        return true;
    }

    // `marks` (host timelines): 1 + 3 * rounds timing events: the start,
    // then per round its frames in, decoded, outputs out
    ZL_Report enqueueHost(const void* hIn, void* hOut, cudaStream_t s, const std::vector<cudaEvent_t>* marks = nullptr)
    {
        size_t const nr = host.rounds.size();
        uint8_t* const dIn = const_cast<uint8_t*>(dFrames[0]);
        uint32_t* const st = reinterpret_cast<uint32_t*>(status.data());
        bool ok = cudaMemsetAsync(st, 0, 4, s) == cudaSuccess && cudaEventRecord(host.start, s) == cudaSuccess
                  && cudaStreamWaitEvent(host.sIn, host.start, 0) == cudaSuccess
                  && cudaStreamWaitEvent(host.sOut, host.start, 0) == cudaSuccess;
        for (size_t r = 0; r < nr && ok; r++) {
            size_t const a = host.inOff[r], b = host.inOff[r + 1];
            if (b > a)
                ok = cudaMemcpyAsync(dIn + a, static_cast<const uint8_t*>(hIn) + a, b - a, cudaMemcpyHostToDevice,
                                     host.sIn) == cudaSuccess;
            ok = ok && cudaEventRecord(host.inEv[r], host.sIn) == cudaSuccess;
            if (marks) cudaEventRecord((*marks)[1 + 3 * r], host.sIn);
        }
        if (marks) cudaEventRecord((*marks)[0], s);
        for (size_t r = 0; r < nr && ok; r++) {
            Part& p = host.rounds[r];
            // at most hostDepth rounds decode at once: round r waits for round r - depth
            if (hostDepth > 0 && r >= size_t(hostDepth))
                ok = cudaStreamWaitEvent(host.rs[r], host.decEv[r - size_t(hostDepth)], 0) == cudaSuccess;
            ok = ok && cudaStreamWaitEvent(host.rs[r], host.inEv[r], 0) == cudaSuccess
                 && runLaunches(p.layout, p.pool.data(), p.scratch.data(), st, host.rs[r]) >= 0
                 && cudaEventRecord(host.decEv[r], host.rs[r]) == cudaSuccess;
            if (marks) cudaEventRecord((*marks)[2 + 3 * r], host.rs[r]);
        }
        for (size_t r = 0; r < nr && ok; r++) {
            size_t const a = host.outOff[r], b = host.outOff[r + 1];
            ok = cudaStreamWaitEvent(host.sOut, host.decEv[r], 0) == cudaSuccess;
            if (ok && b > a)
                ok = cudaMemcpyAsync(static_cast<uint8_t*>(hOut) + a, dOuts[0] + a, b - a, cudaMemcpyDeviceToHost,
                                     host.sOut) == cudaSuccess;
            if (marks) cudaEventRecord((*marks)[3 + 3 * r], host.sOut);
        }
        ok = ok && cudaEventRecord(host.outDone, host.sOut) == cudaSuccess
             && cudaStreamWaitEvent(s, host.outDone, 0) == cudaSuccess
             && cudaStreamWaitEvent(s, host.inEv[nr - 1], 0) == cudaSuccess;
        for (size_t r = 0; r < nr && ok; r++) ok = cudaStreamWaitEvent(s, host.decEv[r], 0) == cudaSuccess;
        if (!ok) {
            err = std::string("host pipeline launch failed: ") + cudaGetErrorString(cudaGetLastError());
            return reportFail(ZL_ErrorCode_GENERIC);
        }
        return reportOk(0);
    }

    // Copies the frames in from hIn, decodes and copies the outputs out to
    // hOut, overlapped by rounds when the frames are laid out in order.
    ZL_Report runHost(const void* hIn, size_t inBytes, void* hOut, size_t outBytes, cudaStream_t s, bool useGraph)
    {
        if (!buildRounds(inBytes, outBytes)) {
            cudaError_t e = inBytes ? cudaMemcpyAsync(const_cast<uint8_t*>(dFrames[0]), hIn, inBytes,
                                                      cudaMemcpyHostToDevice, s)
                                    : cudaSuccess;
            if (e != cudaSuccess) {
                err = std::string("frame upload failed: ") + cudaGetErrorString(e);
                return reportFail(ZL_ErrorCode_GENERIC);
            }
            ZL_Report r = run(s, useGraph);
            if (ZL_isError(r)) return r;
            e = outBytes ? cudaMemcpyAsync(hOut, dOuts[0], outBytes, cudaMemcpyDeviceToHost, s) : cudaSuccess;
            if (e != cudaSuccess) {
                err = std::string("output download failed: ") + cudaGetErrorString(e);
                return reportFail(ZL_ErrorCode_GENERIC);
            }
            return check(s);
        }
        ZL_Report u = upload(s);
        if (ZL_isError(u)) return u;
        if (!host.uploaded) {
            afterLastRun(s);
            for (Part& p : host.rounds) {
                if (p.layout.pool.empty()) continue;
                cudaError_t const e = cudaMemcpyAsync(p.pool.data(), p.layout.pool.data(), p.layout.pool.size(),
                                                      cudaMemcpyHostToDevice, s);
                if (e != cudaSuccess) {
                    err = std::string("round descriptor upload failed: ") + cudaGetErrorString(e);
                    return reportFail(ZL_ErrorCode_GENERIC);
                }
            }
            host.uploaded = true;
        }
        if (!useGraph) {
            ZL_Report r = enqueueHost(hIn, hOut, s);
            if (ZL_isError(r)) return r;
            markRun(s);
            return check(s);
        }
        if (s == nullptr) {
            err = "CUDA graph capture needs a non-default stream";
            return reportFail(ZL_ErrorCode_parameter_invalid);
        }
        if (!host.graph || host.gIn != hIn || host.gOut != hOut || host.gInBytes != inBytes || host.gOutBytes != outBytes
            || host.gStream != s) {
            host.dropGraph();
            cudaGraph_t g = nullptr;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
                err = "stream capture failed";
                return reportFail(ZL_ErrorCode_GENERIC);
            }
            ZL_Report r = enqueueHost(hIn, hOut, s);
            cudaError_t e = cudaStreamEndCapture(s, &g);
            if (ZL_isError(r)) { if (g) cudaGraphDestroy(g); return r; }
            if (e != cudaSuccess) { err = "stream capture failed"; return reportFail(ZL_ErrorCode_GENERIC); }
            e = cudaGraphInstantiateWithFlags(&host.graph, g, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { host.graph = nullptr; err = "graph instantiation failed"; return reportFail(ZL_ErrorCode_GENERIC); }
            host.gIn = hIn;
            host.gOut = hOut;
            host.gInBytes = inBytes;
            host.gOutBytes = outBytes;
            host.gStream = s;
        }
        if (cudaGraphLaunch(host.graph, s) != cudaSuccess) { err = "graph launch failed"; return reportFail(ZL_ErrorCode_GENERIC); }
        markRun(s);
        return check(s);
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
