// Serving loop: continuous batching of decompress and compress requests on
// one GPU (ozl_server_* in include/openzl_gb300.h; no counterpart in the
// reference, which compresses one frame per call on the CPU).
//
// Requests queue on the host. The server holds one resident device pool of
// the HBM budget, shared by its workers; each worker thread owns a CUDA
// stream and its own decode and encode engines. A free worker admits the
// oldest queued request and the next ones of the same kind, as many as fit
// one contiguous block of the pool (at most the budget's per-worker share,
// unless the oldest request alone is larger), copies them in, runs them as
// one batch, copies the results out, returns the block and reports each
// request's latency. Admission waits for free HBM, not for a free worker's
// fixed arena: a request up to the whole budget runs as soon as enough of the
// pool is free, and only a request larger than the budget is refused. Workers
// run their batches concurrently, so requests that arrive while others are on
// the GPU are admitted as soon as a worker and memory free up, and their work
// overlaps on the device. Codec work is bit-exact and per frame, so a result
// does not depend on the batch it ran in.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/openzl_gb300.h"
#include "decode_batch.h"
#include "enc_engine.h"
#include "pool_blocks.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr size_t kAlign = 256;
size_t alignUp(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

struct Request {
    uint64_t id;
    int kind; // 0 decompress, 1 compress
    const uint8_t* in;
    size_t inBytes;
    size_t nbElts;   // compress
    int width;       // compress: 0 serial, else element width
    int recipe;      // compress
    uint8_t* out;
    size_t outCap;
    size_t outBytes; // decompress: decoded size; compress: device bound
    Clock::time_point t0;
    ZL_Report result;
    double latencyUs;
};

} // namespace

struct OZL_Server_s {
    int device = 0;
    size_t budget = 0;     // bytes of the shared pool
    size_t share = 0;      // batch size cap: the budget's per-worker share
    ozl::DevBuf pool;
    ozl::PoolBlocks blocks;
    int nbWorkers = 0;
    int checksums = 1;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<Request*> pending;
    std::deque<Request*> done;
    std::vector<std::thread> workers;
    uint64_t nextId = 1;
    bool stop = false;
    size_t inFlight = 0;
    // cumulative per-stage times of the workers (ozl_server_stats), under mu
    enum { ST_DEC_BATCHES, ST_DEC_REQS, ST_DEC_PLAN, ST_DEC_RUN, ST_ENC_BATCHES, ST_ENC_REQS, ST_ENC_RUN, ST_WAIT,
           ST_COUNT };
    double stats[ST_COUNT] = {};
    void addStat(int k, double v)
    {
        std::lock_guard<std::mutex> lk(mu);
        stats[k] += v;
    }

    void worker();
    void runDecode(std::vector<Request*>& batch, ozl::DecodeBatch& dec, uint8_t* arena, cudaStream_t s);
    void runEncode(std::vector<Request*>& batch, ozl::EncodeBatch& enc, uint8_t* arena, cudaStream_t s);
    void finish(std::vector<Request*>& batch)
    {
        Clock::time_point const t = Clock::now();
        std::lock_guard<std::mutex> lk(mu);
        for (Request* r : batch) {
            r->latencyUs = std::chrono::duration<double, std::micro>(t - r->t0).count();
            done.push_back(r);
        }
        inFlight -= batch.size();
        cvDone.notify_all();
    }
    void finishOne(Request* r)
    {
        std::vector<Request*> one{ r };
        finish(one);
    }
};

void OZL_Server_s::worker()
{
    cudaSetDevice(device);
    cudaStream_t s = nullptr;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    ozl::DecodeBatch dec;
    ozl::EncodeBatch enc;
    dec.checkContent = dec.checkCompressed = checksums != 0;
    // the encoder's parallel host phases and the decode plans on this
    // worker's share of the cores
    unsigned const hw = std::thread::hardware_concurrency();
    unsigned const cores = std::max(2u, (hw ? hw : 16u) / unsigned(nbWorkers));
    enc.setHostThreads(cores);
    dec.planThreads = cores;
    auto need = [](const Request* r) { return alignUp(r->inBytes) + alignUp(r->outBytes); };
    for (;;) {
        std::vector<Request*> batch;
        size_t off = 0, bytes = 0;
        Clock::time_point const tIdle = Clock::now();
        {
            std::unique_lock<std::mutex> lk(mu);
            // the oldest request is admitted when a block of its size is free
            // (or refused at once when it exceeds the whole budget)
            cvWork.wait(lk, [&] {
                if (stop && pending.empty()) return true;
                if (pending.empty()) return false;
                size_t const n = need(pending.front());
                return n > budget || blocks.largest() >= n;
            });
            if (pending.empty() && stop) break;
            Request* head = pending.front();
            size_t const headNeed = need(head);
            if (headNeed > budget) {
                pending.pop_front();
                head->result = ozl::reportFail(ZL_ErrorCode_srcSize_tooLarge);
                lk.unlock();
                finishOne(head);
                continue;
            }
            // then the next requests of the same kind, oldest first, while the
            // batch fits the largest free block and the per-worker share
            size_t const cap = std::min(blocks.largest(), std::max(share, headNeed));
            int const kind = head->kind;
            for (auto it = pending.begin(); it != pending.end();) {
                Request* r = *it;
                if (r->kind != kind) { ++it; continue; }
                size_t const n = need(r);
                if (bytes + n > cap) break;
                bytes += n;
                batch.push_back(r);
                it = pending.erase(it);
            }
            blocks.take(bytes, off); // fits: bytes <= the largest free block
            if (!pending.empty()) cvWork.notify_one(); // another worker may admit the rest
            stats[ST_WAIT] += std::chrono::duration<double>(Clock::now() - tIdle).count();
        }
        if (!pool.data() || !s) {
            for (Request* r : batch) r->result = ozl::reportFail(ZL_ErrorCode_allocation);
        } else if (batch.front()->kind == 0) {
            runDecode(batch, dec, pool.data() + off, s);
        } else {
            runEncode(batch, enc, pool.data() + off, s);
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            blocks.give(off, bytes);
        }
        cvWork.notify_all(); // freed memory may admit waiting requests
        finish(batch);
    }
    if (s) cudaStreamDestroy(s);
}

void OZL_Server_s::runDecode(std::vector<Request*>& batch, ozl::DecodeBatch& dec, uint8_t* arena, cudaStream_t s)
{
    size_t const n = batch.size();
    std::vector<const void*> hF(n), dF(n);
    std::vector<void*> dO(n);
    std::vector<size_t> fs(n), caps(n);
    size_t pos = 0;
    for (size_t i = 0; i < n; i++) {
        Request* r = batch[i];
        hF[i] = r->in;
        fs[i] = r->inBytes;
        dF[i] = arena + pos;
        pos += alignUp(r->inBytes);
        dO[i] = arena + pos;
        caps[i] = r->outBytes;
        pos += alignUp(r->outBytes);
        cudaMemcpyAsync(const_cast<void*>(dF[i]), r->in, r->inBytes, cudaMemcpyHostToDevice, s);
    }
    Clock::time_point const t0 = Clock::now();
    ZL_Report rep = dec.makePlan(n, hF.data(), fs.data(), dF.data(), dO.data(), caps.data());
    Clock::time_point const t1 = Clock::now();
    if (!ZL_isError(rep)) rep = dec.run(s, false);
    if (!ZL_isError(rep)) rep = dec.check(s);
    {
        std::lock_guard<std::mutex> lk(mu);
        stats[ST_DEC_BATCHES] += 1;
        stats[ST_DEC_REQS] += double(n);
        stats[ST_DEC_PLAN] += std::chrono::duration<double>(t1 - t0).count();
        stats[ST_DEC_RUN] += std::chrono::duration<double>(Clock::now() - t1).count();
    }
    if (ZL_isError(rep) && n > 1) {
        // attribute the error: each frame alone
        for (size_t i = 0; i < n; i++) {
            std::vector<Request*> one{ batch[i] };
            runDecode(one, dec, arena, s);
        }
        return;
    }
    for (size_t i = 0; i < n; i++) {
        Request* r = batch[i];
        if (ZL_isError(rep)) { r->result = rep; continue; }
        if (r->outBytes > r->outCap) { r->result = ozl::reportFail(ZL_ErrorCode_dstCapacity_tooSmall); continue; }
        if (r->outBytes) cudaMemcpyAsync(r->out, dO[i], r->outBytes, cudaMemcpyDeviceToHost, s);
        r->result = ozl::reportOk(r->outBytes);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
        for (Request* r : batch) r->result = ozl::reportFail(ZL_ErrorCode_GENERIC);
}

void OZL_Server_s::runEncode(std::vector<Request*>& batch, ozl::EncodeBatch& enc, uint8_t* arena, cudaStream_t s)
{
    size_t const n = batch.size();
    std::vector<ozl::EncFrameSpec> specs(n);
    std::vector<uint8_t*> dOut(n);
    std::vector<size_t> caps(n);
    size_t pos = 0;
    for (size_t i = 0; i < n; i++) {
        Request* r = batch[i];
        uint8_t* dIn = arena + pos;
        pos += alignUp(r->inBytes);
        dOut[i] = arena + pos;
        caps[i] = r->outBytes;
        pos += alignUp(r->outBytes);
        if (r->inBytes) cudaMemcpyAsync(dIn, r->in, r->inBytes, cudaMemcpyHostToDevice, s);
        specs[i] = ozl::EncFrameSpec{ dIn, r->nbElts, uint32_t(r->width ? r->width : 1), r->width == 0, r->recipe };
    }
    std::vector<size_t> sizes;
    std::string err;
    Clock::time_point const t0 = Clock::now();
    int rc = enc.compress(specs, dOut.data(), caps.data(), checksums != 0, s, sizes, err);
    {
        std::lock_guard<std::mutex> lk(mu);
        stats[ST_ENC_BATCHES] += 1;
        stats[ST_ENC_REQS] += double(n);
        stats[ST_ENC_RUN] += std::chrono::duration<double>(Clock::now() - t0).count();
    }
    if (rc && n > 1) {
        for (size_t i = 0; i < n; i++) {
            std::vector<Request*> one{ batch[i] };
            runEncode(one, enc, arena, s);
        }
        return;
    }
    for (size_t i = 0; i < n; i++) {
        Request* r = batch[i];
        if (rc) { r->result = ozl::reportFail(rc); continue; }
        if (sizes[i] > r->outCap) { r->result = ozl::reportFail(ZL_ErrorCode_dstCapacity_tooSmall); continue; }
        cudaMemcpyAsync(r->out, dOut[i], sizes[i], cudaMemcpyDeviceToHost, s);
        r->result = ozl::reportOk(sizes[i]);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
        for (Request* r : batch) r->result = ozl::reportFail(ZL_ErrorCode_GENERIC);
}

extern "C" {

size_t ozl_server_stats(OZL_Server* srv, double* out, size_t capacity)
{
    if (!srv) return 0;
    std::lock_guard<std::mutex> lk(srv->mu);
    for (size_t i = 0; i < capacity && i < size_t(OZL_Server_s::ST_COUNT); i++) out[i] = srv->stats[i];
    return size_t(OZL_Server_s::ST_COUNT);
}

OZL_Server* ozl_server_create(size_t hbmBudget, int nbWorkers, int checksums)
{
    if (nbWorkers < 1 || nbWorkers > 64 || hbmBudget < size_t(nbWorkers) * (1u << 20)) return nullptr;
    OZL_Server_s* srv = new (std::nothrow) OZL_Server_s();
    if (!srv) return nullptr;
    if (cudaGetDevice(&srv->device) != cudaSuccess) {
        delete srv;
        return nullptr;
    }
    srv->nbWorkers = nbWorkers;
    srv->budget = hbmBudget / kAlign * kAlign;
    srv->share = hbmBudget / size_t(nbWorkers) / kAlign * kAlign;
    srv->checksums = checksums;
    if (!srv->pool.reserve(srv->budget)) {
        delete srv;
        return nullptr;
    }
    srv->blocks.reset(srv->budget);
    try {
        for (int i = 0; i < nbWorkers; i++) srv->workers.emplace_back([srv] { srv->worker(); });
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->stop = true;
        }
        srv->cvWork.notify_all();
        for (auto& t : srv->workers) t.join();
        delete srv;
        return nullptr;
    }
    return srv;
}

void ozl_server_free(OZL_Server* srv)
{
    if (!srv) return;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cvWork.notify_all();
    for (auto& t : srv->workers) t.join();
    for (Request* r : srv->done) delete r;
    for (Request* r : srv->pending) delete r;
    delete srv;
}

static uint64_t enqueue(OZL_Server* srv, Request* r)
{
    std::lock_guard<std::mutex> lk(srv->mu);
    r->id = srv->nextId++;
    srv->pending.push_back(r);
    srv->inFlight++;
    srv->cvWork.notify_one();
    return r->id;
}

uint64_t ozl_server_submit_decompress(OZL_Server* srv, const void* frame, size_t frameSize, void* dst,
                                      size_t dstCapacity)
{
    if (!srv || !frame) return 0;
    Request* r = new (std::nothrow) Request{};
    if (!r) return 0;
    r->t0 = Clock::now();
    r->kind = 0;
    r->in = static_cast<const uint8_t*>(frame);
    r->inBytes = frameSize;
    r->out = static_cast<uint8_t*>(dst);
    r->outCap = dstCapacity;
    ZL_Report ds = ozl::singleOutputSize(frame, frameSize);
    if (ZL_isError(ds)) { // answered at once, never queued
        uint64_t id;
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            id = r->id = srv->nextId++;
            srv->inFlight++;
        }
        r->result = ds;
        srv->finishOne(r);
        return id;
    }
    r->outBytes = ZL_validResult(ds);
    return enqueue(srv, r);
}

uint64_t ozl_server_submit_compress(OZL_Server* srv, const void* src, size_t nbElts, int eltWidth, int recipe,
                                    void* dst, size_t dstCapacity)
{
    if (!srv || (nbElts && !src) || !(eltWidth == 0 || eltWidth == 1 || eltWidth == 2 || eltWidth == 4 || eltWidth == 8))
        return 0;
    Request* r = new (std::nothrow) Request{};
    if (!r) return 0;
    r->t0 = Clock::now();
    r->kind = 1;
    r->in = static_cast<const uint8_t*>(src);
    r->inBytes = nbElts * size_t(eltWidth ? eltWidth : 1);
    r->nbElts = nbElts;
    r->width = eltWidth;
    r->recipe = recipe;
    r->out = static_cast<uint8_t*>(dst);
    r->outCap = dstCapacity;
    r->outBytes = ozl::encodeBound(r->inBytes);
    return enqueue(srv, r);
}

size_t ozl_server_poll(OZL_Server* srv, uint64_t* ids, ZL_Report* results, double* latencyUs, size_t max,
                       int waitMs)
{
    if (!srv || max == 0) return 0;
    std::unique_lock<std::mutex> lk(srv->mu);
    if (srv->done.empty() && waitMs > 0)
        srv->cvDone.wait_for(lk, std::chrono::milliseconds(waitMs), [&] { return !srv->done.empty(); });
    size_t k = 0;
    while (k < max && !srv->done.empty()) {
        Request* r = srv->done.front();
        srv->done.pop_front();
        if (ids) ids[k] = r->id;
        if (results) results[k] = r->result;
        if (latencyUs) latencyUs[k] = r->latencyUs;
        delete r;
        k++;
    }
    return k;
}

size_t ozl_server_in_flight(OZL_Server* srv)
{
    if (!srv) return 0;
    std::lock_guard<std::mutex> lk(srv->mu);
    return srv->inFlight;
}

} // extern "C"
