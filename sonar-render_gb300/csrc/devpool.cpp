// devpool.cpp -- one stream-ordered memory pool per GPU for every device
// buffer the library owns (fragment data, masks, compressed blocks, work
// lists, batch plans).
//
// cudaMalloc maps new pages and cudaFree waits for the whole device, so a
// scene that is torn down and loaded again (the reference's TearDownCuda /
// load / render cycle) paid for both on every call.  Blocks from a pool that
// keeps freed memory come back without either: cudaMallocFromPoolAsync and
// cudaFreeAsync are ordered on the stream that uses the block, and the pool's
// own reuse rules (event dependencies between streams) make a block freed on
// one stream safe to hand out on another.  Memory above the cache limit goes
// back to the device at the next synchronisation.
//
// Host <-> device copies of the library's own arrays go through two pinned
// chunks: a copy from pageable memory runs at a few GB/s on the host side,
// one from pinned memory at the link's rate, so the host fills (or drains)
// one chunk while the other is on the link.
#include "devpool.h"
#include "host.h"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

namespace sonar {

namespace {

constexpr int kMaxDevices = 64;
cudaMemPool_t g_pools[kMaxDevices] = {};
unsigned long long g_limit = 32ull << 30;  // unused bytes kept per pool
std::mutex g_mu;

cudaMemPool_t current_pool(cudaError_t *err)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess && (dev < 0 || dev >= kMaxDevices)) e = cudaErrorInvalidDevice;
    if (e != cudaSuccess) {
        *err = e;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps pr{};
        pr.allocType = cudaMemAllocationTypePinned;
        pr.location.type = cudaMemLocationTypeDevice;
        pr.location.id = dev;
        cudaMemPool_t p = nullptr;
        e = cudaMemPoolCreate(&p, &pr);
        if (e == cudaSuccess) {
            unsigned long long th = g_limit;
            e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &th);
            if (e != cudaSuccess) cudaMemPoolDestroy(p);
        }
        if (e != cudaSuccess) {
            *err = e;
            return nullptr;
        }
        g_pools[dev] = p;
    }
    return g_pools[dev];
}

}  // namespace

cudaError_t pool_alloc(void **out, size_t bytes, cudaStream_t s)
{
    *out = nullptr;
    cudaError_t e = cudaSuccess;
    cudaMemPool_t p = current_pool(&e);
    if (!p) return e;
    if (bytes == 0) bytes = 1;
    e = cudaMallocFromPoolAsync(out, bytes, p, s);
    if (e == cudaErrorMemoryAllocation) {
        // the pool may hold enough memory in blocks of other sizes: wait for
        // every pending free, give the unused memory back, try once more
        (void)cudaGetLastError();
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemPoolTrimTo(p, 0);
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(out, bytes, p, s);
    }
    if (e != cudaSuccess) {
        (void)cudaGetLastError();  // an allocation failure leaves the context usable
        *out = nullptr;
    }
    return e;
}

void pool_free(void *ptr, cudaStream_t s)
{
    if (ptr) (void)cudaFreeAsync(ptr, s);
}

void pool_set_cache_limit(unsigned long long bytes)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_limit = bytes;
    for (cudaMemPool_t p : g_pools)
        if (p) {
            unsigned long long th = bytes;
            (void)cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &th);
        }
}

unsigned long long pool_cache_limit()
{
    std::lock_guard<std::mutex> lk(g_mu);
    return g_limit;
}

cudaError_t pool_trim()
{
    cudaError_t e = cudaDeviceSynchronize();
    std::lock_guard<std::mutex> lk(g_mu);
    for (cudaMemPool_t p : g_pools)
        if (p && e == cudaSuccess) e = cudaMemPoolTrimTo(p, 0);
    return e;
}

unsigned long long pool_reserved_bytes()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 0;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_pools[dev]) return 0;
    unsigned long long v = 0;
    if (cudaMemPoolGetAttribute(g_pools[dev], cudaMemPoolAttrReservedMemCurrent, &v) != cudaSuccess) return 0;
    return v;
}

namespace {

constexpr size_t kStageChunk = 8u << 20;
constexpr size_t kStageDirect = 256u << 10;

struct Stage {
    char *buf[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    bool pending[2] = {false, false};
    int next = 0;  // chunk the next upload fills (successive calls alternate)
    int dev = -1;
};
Stage g_stage;
std::mutex g_stage_mu;

// Pinned chunks (kept for the process) and their events on the current device.
bool stage_ready(Stage &st)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (st.buf[0] && st.dev == dev) return true;
    for (int b = 0; b < 2; b++) {
        if (st.done[b]) {
            if (st.pending[b]) cudaEventSynchronize(st.done[b]);
            cudaEventDestroy(st.done[b]);
            st.done[b] = nullptr;
        }
        st.pending[b] = false;
        if (!st.buf[b] && cudaHostAlloc((void **)&st.buf[b], kStageChunk, cudaHostAllocPortable) != cudaSuccess) {
            st.buf[b] = nullptr;
            (void)cudaGetLastError();
            return false;
        }
        if (cudaEventCreateWithFlags(&st.done[b], cudaEventDisableTiming) != cudaSuccess) {
            st.done[b] = nullptr;
            (void)cudaGetLastError();
            return false;
        }
    }
    st.dev = dev;
    return true;
}

// memcpy on the host workers for large copies (the caller's pages, often
// fresh, fault in on several threads at once)
void host_copy(void *dst, const void *src, size_t n)
{
    constexpr size_t kPiece = 512u << 10;
    if (n < 2 * kPiece) {
        memcpy(dst, src, n);
        return;
    }
    const long long pieces = (long long)((n + kPiece - 1) / kPiece);
    parallel_units(pieces, [&](long long u) {
        const size_t off = (size_t)u * kPiece;
        memcpy((char *)dst + off, (const char *)src + off, std::min(kPiece, n - off));
    });
}

// Waits until chunk b's last copy is done.
cudaError_t stage_wait(Stage &st, int b)
{
    if (!st.pending[b]) return cudaSuccess;
    st.pending[b] = false;
    return cudaEventSynchronize(st.done[b]);
}

}  // namespace

cudaError_t stage_to_device(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    if (bytes == 0) return cudaSuccess;
    std::unique_lock<std::mutex> lk(g_stage_mu);
    if (bytes < kStageDirect || !stage_ready(g_stage)) {
        lk.unlock();
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
    }
    Stage &st = g_stage;
    for (size_t off = 0; off < bytes; off += kStageChunk) {
        const int b = st.next;
        st.next ^= 1;
        const size_t n = std::min(kStageChunk, bytes - off);
        cudaError_t e = stage_wait(st, b);
        if (e != cudaSuccess) return e;
        host_copy(st.buf[b], (const char *)src + off, n);
        e = cudaMemcpyAsync((char *)dst + off, st.buf[b], n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaEventRecord(st.done[b], s);
        if (e != cudaSuccess) return e;
        st.pending[b] = true;
    }
    return cudaSuccess;
}

cudaError_t stage_to_host(void *dst, const void *src, size_t bytes, cudaStream_t s)
{
    if (bytes == 0) return cudaSuccess;
    std::unique_lock<std::mutex> lk(g_stage_mu);
    if (bytes < kStageDirect || !stage_ready(g_stage)) {
        lk.unlock();
        cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
    }
    Stage &st = g_stage;
    const size_t nch = (bytes + kStageChunk - 1) / kStageChunk;
    auto issue = [&](size_t k) {
        const int b = (int)(k & 1);
        const size_t off = k * kStageChunk, n = std::min(kStageChunk, bytes - off);
        cudaError_t e = stage_wait(st, b);
        if (e == cudaSuccess) e = cudaMemcpyAsync(st.buf[b], (const char *)src + off, n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaEventRecord(st.done[b], s);
        if (e == cudaSuccess) st.pending[b] = true;
        return e;
    };
    cudaError_t e = issue(0);
    if (e == cudaSuccess && nch > 1) e = issue(1);
    for (size_t k = 0; k < nch && e == cudaSuccess; k++) {
        const int b = (int)(k & 1);
        const size_t off = k * kStageChunk, n = std::min(kStageChunk, bytes - off);
        e = stage_wait(st, b);
        if (e != cudaSuccess) break;
        host_copy((char *)dst + off, st.buf[b], n);
        if (k + 2 < nch) e = issue(k + 2);
    }
    return e;
}

namespace {

struct HostBlock {
    char *p = nullptr;
    size_t cap = 0, used = 0;
};
std::vector<HostBlock> g_host_blocks;
size_t g_host_want = 0;  // one block of this size after a reset that found several
std::mutex g_host_mu;

}  // namespace

void *host_arena_take(size_t bytes)
{
    std::lock_guard<std::mutex> lk(g_host_mu);
    bytes = (std::max<size_t>(bytes, 1) + 255) / 256 * 256;
    if (!g_host_blocks.empty()) {
        HostBlock &b = g_host_blocks.back();
        if (b.used + bytes <= b.cap) {
            void *r = b.p + b.used;
            b.used += bytes;
            return r;
        }
    }
    size_t total = 0;
    for (const HostBlock &b : g_host_blocks) total += b.cap;
    HostBlock nb;
    nb.cap = std::max({bytes, 2 * total, g_host_want, (size_t)32 << 20});
    if (cudaHostAlloc((void **)&nb.p, nb.cap, cudaHostAllocPortable) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    g_host_want = 0;
    nb.used = bytes;
    g_host_blocks.push_back(nb);
    return nb.p;
}

void host_arena_reset()
{
    std::lock_guard<std::mutex> lk(g_host_mu);
    if (g_host_blocks.size() > 1) {
        // several blocks: the next take allocates one block holding them all
        size_t total = 0;
        for (HostBlock &b : g_host_blocks) {
            total += b.cap;
            cudaFreeHost(b.p);
        }
        g_host_blocks.clear();
        g_host_want = total;
    } else if (!g_host_blocks.empty()) {
        g_host_blocks[0].used = 0;
    }
}

}  // namespace sonar
