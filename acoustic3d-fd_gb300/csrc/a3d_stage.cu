// a3d_stage.cu — model uploads from pageable caller memory.
//
// A cudaMemcpy from pageable memory makes the driver pin the caller's pages for
// every call; on the Grace host that ran at 3.5-5 GB/s for a 151 MB model array
// once a process had run a few engines (against 130-190 GB/s from pinned memory).
// Uploads go through a pinned staging ring instead, allocated on first use and
// kept for the life of the process: host threads copy one chunk of the caller's
// buffer into a slot while the copy engine moves the previous chunk, so both run
// at once.  Calls take a process-wide lock (one upload at a time uses the ring);
// if the ring cannot be allocated, the plain copy runs.  Record downloads into a
// caller's array stay plain copies: through the ring they were no faster (17-32
// GB/s against 26-28), the caller's fresh destination pages being what limits
// them.  Downloads that end in a file (the legacy entry points' shot records) go
// through the ring instead (stage_from_device): the copy engine fills one slot
// while host threads write the previous one to the file, so the file never waits
// for a whole-record copy and no pageable copy of the record is made.
#include <algorithm>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "a3d_engine.h"

namespace a3d {

namespace {

constexpr size_t STAGE_CHUNK = size_t(32) << 20;  // bytes per slot
constexpr int STAGE_SLOTS = 3;
constexpr size_t STAGE_MIN = size_t(4) << 20;     // smaller copies go straight through

std::mutex g_stage_mu;
unsigned char *g_stage = nullptr;  // STAGE_SLOTS * STAGE_CHUNK pinned bytes
bool g_stage_failed = false;

unsigned char *stage_ring() {  // under g_stage_mu
    if (!g_stage && !g_stage_failed) {
        void *p = nullptr;
        if (cudaHostAlloc(&p, STAGE_SLOTS * STAGE_CHUNK, cudaHostAllocPortable) == cudaSuccess) {
            g_stage = static_cast<unsigned char *>(p);
        } else {
            g_stage_failed = true;
            cudaGetLastError();
        }
    }
    return g_stage;
}

// memcpy of n bytes over up to 4 host threads (this one included)
void par_copy(unsigned char *dst, const unsigned char *src, size_t n) {
    const size_t nth = n >= (size_t(8) << 20) ? std::min<size_t>(4, std::max(1u, std::thread::hardware_concurrency())) : 1;
    const size_t part = (n / nth + 4095) & ~size_t(4095);
    std::vector<std::thread> ts;
    size_t next = std::min(n, part);  // this thread copies [0, part)
    try {
        while (next < n) {
            const size_t len = std::min(part, n - next);
            ts.emplace_back([=] { memcpy(dst + next, src + next, len); });
            next += len;
        }
    } catch (...) {  // a thread could not be started: this thread copies what is left
    }
    memcpy(dst, src, std::min(n, part));
    if (next < n) memcpy(dst + next, src + next, n - next);
    for (auto &t : ts) t.join();
}

struct Events {
    cudaEvent_t ev[STAGE_SLOTS] = {};
    cudaError_t make() {
        for (auto &e : ev) {
            const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    }
    ~Events() {
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
};

}  // namespace

int stage_to_device(void *dst, const void *src, size_t bytes, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_stage_mu);
    unsigned char *ring = bytes >= STAGE_MIN ? stage_ring() : nullptr;
    cudaError_t r = cudaSuccess;
    if (!ring) {
        r = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
        if (r == cudaSuccess) r = cudaStreamSynchronize(st);
    } else {
        Events ev;
        r = ev.make();
        const unsigned char *s = static_cast<const unsigned char *>(src);
        unsigned char *d = static_cast<unsigned char *>(dst);
        for (size_t off = 0, k = 0; off < bytes && r == cudaSuccess; off += STAGE_CHUNK, ++k) {
            const int slot = (int)(k % STAGE_SLOTS);
            const size_t n = std::min(STAGE_CHUNK, bytes - off);
            unsigned char *buf = ring + slot * STAGE_CHUNK;
            if (k >= (size_t)STAGE_SLOTS) r = cudaEventSynchronize(ev.ev[slot]);  // the slot's last copy is done
            if (r != cudaSuccess) break;
            par_copy(buf, s + off, n);
            r = cudaMemcpyAsync(d + off, buf, n, cudaMemcpyHostToDevice, st);
            if (r == cudaSuccess) r = cudaEventRecord(ev.ev[slot], st);
        }
        const cudaError_t r2 = cudaStreamSynchronize(st);  // no slot is in use on return
        if (r == cudaSuccess) r = r2;
    }
    if (r != cudaSuccess) return fail(A3D_E_CUDA, "host-to-device copy of %zu bytes failed: %s", bytes, cudaGetErrorString(r));
    return A3D_OK;
}

int stage_from_device(const void *src, size_t bytes, cudaStream_t st,
                      const std::function<int(const unsigned char *, size_t, size_t)> &sink) {
    std::lock_guard<std::mutex> lk(g_stage_mu);
    unsigned char *ring = stage_ring();
    const unsigned char *s = static_cast<const unsigned char *>(src);
    const size_t nchunks = (bytes + STAGE_CHUNK - 1) / STAGE_CHUNK;
    cudaError_t r = cudaSuccess;
    if (!ring) {  // no pinned ring: plain copies, one chunk at a time
        std::vector<unsigned char> buf(std::min(bytes, STAGE_CHUNK));
        for (size_t k = 0; k < nchunks; ++k) {
            const size_t off = k * STAGE_CHUNK, n = std::min(STAGE_CHUNK, bytes - off);
            if ((r = cudaMemcpyAsync(buf.data(), s + off, n, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (r = cudaStreamSynchronize(st)) != cudaSuccess)
                break;
            const int rc = sink(buf.data(), off, n);
            if (rc) return rc;
        }
    } else {
        Events ev;
        r = ev.make();
        auto issue = [&](size_t k) -> cudaError_t {
            const int slot = (int)(k % STAGE_SLOTS);
            const size_t off = k * STAGE_CHUNK, n = std::min(STAGE_CHUNK, bytes - off);
            cudaError_t e = cudaMemcpyAsync(ring + slot * STAGE_CHUNK, s + off, n, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaEventRecord(ev.ev[slot], st);
            return e;
        };
        // keep STAGE_SLOTS - 1 copies ahead of the sink; chunk k + SLOTS - 1 reuses the
        // slot of chunk k - 1, which the sink finished with in the previous iteration
        for (size_t k = 0; k + 1 < (size_t)STAGE_SLOTS && k < nchunks && r == cudaSuccess; ++k) r = issue(k);
        int rc = A3D_OK;
        for (size_t k = 0; k < nchunks && r == cudaSuccess && !rc; ++k) {
            if (k + STAGE_SLOTS - 1 < nchunks && (r = issue(k + STAGE_SLOTS - 1)) != cudaSuccess) break;
            const int slot = (int)(k % STAGE_SLOTS);
            if ((r = cudaEventSynchronize(ev.ev[slot])) != cudaSuccess) break;
            const size_t off = k * STAGE_CHUNK;
            rc = sink(ring + slot * STAGE_CHUNK, off, std::min(STAGE_CHUNK, bytes - off));
        }
        const cudaError_t r2 = cudaStreamSynchronize(st);  // no slot is in use on return
        if (r == cudaSuccess) r = r2;
        if (rc) return rc;
    }
    if (r != cudaSuccess) return fail(A3D_E_CUDA, "device-to-host copy of %zu bytes failed: %s", bytes, cudaGetErrorString(r));
    return A3D_OK;
}

}  // namespace a3d
