// noalloc.cu -- shortest-path tree of a caller-owned CSR graph without any device allocation.
//
// Some callers cannot call cudaMalloc at the point where they need a shortest-path tree:
// plugins of inference or stream-processing runtimes whose enqueue callbacks must not
// allocate (the host runtime owns the memory budget and cudaMalloc may synchronize the
// device), and pipelines that reserve all device memory up front.  dsssp_sssp_noalloc()
// serves them: the caller passes the graph and the output arrays in its own device memory,
// and the engine's work space (row descriptors, distance words, frontier tags, work lists,
// control block) comes from one file-scope static device array of fixed size, which every
// GPU that loads the library holds until the process exits.
//
// The computation is the engine's persistent update kernel (update.cu, k_update) in its
// from-scratch mode, the same kernel dsssp_tree_compute() runs.
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/dsssp.h"
#include "engine.cuh"
#include "host_common.h"

namespace dsssp {

cudaError_t update_occupancy(int block, int* blocks_per_sm);
cudaError_t launch_update(const UpdParams& p, int grid, int block, cudaStream_t s);
void count_launch(int n);

namespace {

constexpr long long kMaxV = DSSSP_NOALLOC_MAX_VERTICES;
constexpr long long kMaxE = DSSSP_NOALLOC_MAX_ENTRIES;
constexpr int kTe = 8;        // edges per thread item
constexpr int kLarge = 1024;  // rows above this become CTA items
constexpr int kChunk = 1024;  // edges per CTA item
constexpr int kBlock = 256;
constexpr long long kTcap = kMaxE / kTe + kMaxV + 64;
constexpr long long kCcap = kMaxE / kChunk + kMaxE / kLarge + 64;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCtl = 0;
constexpr size_t kOffRows = align256(kOffCtl + sizeof(Ctl));
constexpr size_t kOffState = align256(kOffRows + sizeof(RowDesc) * kMaxV);
constexpr size_t kOffTag = align256(kOffState + 8 * kMaxV);
constexpr size_t kOffRt0 = align256(kOffTag + 4 * kMaxV);
constexpr size_t kOffRt1 = align256(kOffRt0 + sizeof(Item) * kTcap);
constexpr size_t kOffRc0 = align256(kOffRt1 + sizeof(Item) * kTcap);
constexpr size_t kOffRc1 = align256(kOffRc0 + sizeof(Item) * kCcap);
constexpr size_t kOffSrc = align256(kOffRc1 + sizeof(Item) * kCcap);
constexpr size_t kScratchBytes = align256(kOffSrc + sizeof(int));

// The work space.  Shared by every call on a device; kept between calls.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct DeviceSetup {
    bool done = false;
    unsigned char* base = nullptr;  // device address of g_noalloc_scratch on this device
    int grid = 0;
};

constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

// Clears what must start at zero and fills row descriptors and distance words from the
// caller's CSR; checks the CSR (monotone offsets, ids in range, weights >= 0).
__global__ void k_noalloc_init(unsigned char* base, int n, long long nnz, const long long* off, const int2* adj,
                               int src) {
    Ctl* ctl = reinterpret_cast<Ctl*>(base + kOffCtl);
    RowDesc* rows = reinterpret_cast<RowDesc*>(base + kOffRows);
    unsigned long long* state = reinterpret_cast<unsigned long long*>(base + kOffState);
    unsigned* tag = reinterpret_cast<unsigned*>(base + kOffTag);
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    for (long long v = tid; v < n; v += nthreads) {
        const long long a = off[v], b = off[v + 1];
        RowDesc r;
        r.start = a;
        r.deg = (int)(b - a);
        r.cap = (int)(b - a);
        rows[v] = r;
        state[v] = v == src ? (unsigned long long)(unsigned)src : kInfState;
        tag[v] = 0;
        if (a < 0 || b < a || b > nnz) ctl->diag[7] = 1;  // reported after this kernel
    }
    for (long long e = tid; e < nnz; e += nthreads) {
        const int2 x = adj[e];
        if (x.x < 0 || x.x >= n || x.y < 0) ctl->diag[7] = 1;
    }
}

__global__ void k_noalloc_ctl(unsigned char* base, const long long* off, int n, long long nnz, int src) {
    Ctl* ctl = reinterpret_cast<Ctl*>(base + kOffCtl);
    unsigned* w = reinterpret_cast<unsigned*>(ctl);
    for (unsigned i = threadIdx.x; i < sizeof(Ctl) / 4; i += blockDim.x) w[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        ctl->round_base = 1;
        *reinterpret_cast<int*>(base + kOffSrc) = src;
        if (off[0] != 0 || off[n] != nnz) ctl->diag[7] = 1;
    }
}

// Bad CSR found by k_noalloc_init -> the update kernel sees a non-zero status and skips.
__global__ void k_noalloc_check(unsigned char* base) {
    Ctl* ctl = reinterpret_cast<Ctl*>(base + kOffCtl);
    if (ctl->diag[7]) ctl->status = DSSSP_E_INVAL;
}

__global__ void k_noalloc_out(const unsigned char* base, int n, int* parent, long long* dist) {
    const unsigned long long* state = reinterpret_cast<const unsigned long long*>(base + kOffState);
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const unsigned long long s = state[v];
        parent[v] = s == kInfState ? -1 : (int)(unsigned)s;
        dist[v] = s == kInfState ? DSSSP_UNREACHABLE : (long long)(s >> 32);
    }
}

// Once per device, with that device current: the device address of the scratch array and
// the co-resident grid of the update kernel.
int setup_device(int dev, DeviceSetup** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(DSSSP_E_INVAL, "sssp_noalloc: device %d not supported", dev);
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& s = g_setup[dev];
    if (!s.done) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return fail(DSSSP_E_CUDA, "sssp_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        int per_sm = 0, sms = 0;
        e = update_occupancy(kBlock, &per_sm);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || per_sm < 1)
            return fail(DSSSP_E_COOP, "sssp_noalloc: update kernel has no occupancy (%s)", cudaGetErrorString(e));
        s.base = static_cast<unsigned char*>(ptr);
        s.grid = per_sm * sms;
        s.done = true;
    }
    *out = &s;
    return DSSSP_OK;
}

}  // namespace
}  // namespace dsssp

using namespace dsssp;

extern "C" int dsssp_sssp_noalloc(int32_t n, int64_t nnz, const int64_t* d_row_off, const int32_t* d_adj,
                                  int32_t src, int32_t* d_parent, int64_t* d_dist, void* stream) {
    if (n < 1 || n > kMaxV)
        return fail(DSSSP_E_INVAL, "sssp_noalloc: n=%d outside 1..%lld (DSSSP_NOALLOC_MAX_VERTICES)", n, kMaxV);
    if (nnz < 0 || nnz > kMaxE)
        return fail(DSSSP_E_INVAL, "sssp_noalloc: %lld adjacency entries outside 0..%lld (DSSSP_NOALLOC_MAX_ENTRIES)",
                    (long long)nnz, kMaxE);
    if (src < 0 || src >= n) return fail(DSSSP_E_BAD_VERTEX, "sssp_noalloc: source %d outside 0..%d", src, n - 1);
    // every array is read or written with its natural alignment: a misaligned one would be a
    // device fault, so it is refused here, before any launch
    if (!d_row_off || (nnz > 0 && !d_adj) || !d_parent || !d_dist || ((uintptr_t)d_adj & 7) ||
        ((uintptr_t)d_row_off & 7) || ((uintptr_t)d_dist & 7) || ((uintptr_t)d_parent & 3))
        return fail(DSSSP_E_INVAL, "sssp_noalloc: NULL or misaligned device pointer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(DSSSP_E_NO_DEVICE, "sssp_noalloc: %s", cudaGetErrorString(e));
    DeviceSetup* ds = nullptr;
    int rc = setup_device(dev, &ds);
    if (rc) return rc;
    unsigned char* base = ds->base;
    cudaStream_t s = (cudaStream_t)stream;
    const int2* adj = reinterpret_cast<const int2*>(d_adj);

    k_noalloc_ctl<<<1, 256, 0, s>>>(base, reinterpret_cast<const long long*>(d_row_off), n, nnz, src);
    const long long work = nnz > n ? nnz : n;
    const unsigned blocks = (unsigned)((work + kBlock - 1) / kBlock < 1024 ? (work + kBlock - 1) / kBlock : 1024);
    k_noalloc_init<<<blocks, kBlock, 0, s>>>(base, n, nnz, reinterpret_cast<const long long*>(d_row_off), adj, src);
    k_noalloc_check<<<1, 1, 0, s>>>(base);
    count_launch(3);

    UpdParams p;
    memset(&p, 0, sizeof(p));
    p.g.ctl = reinterpret_cast<Ctl*>(base + kOffCtl);
    p.g.rows = reinterpret_cast<RowDesc*>(base + kOffRows);
    p.g.state = reinterpret_cast<unsigned long long*>(base + kOffState);
    p.g.push_tag = reinterpret_cast<unsigned*>(base + kOffTag);
    p.g.adj = const_cast<int2*>(adj);
    p.g.rt0 = reinterpret_cast<Item*>(base + kOffRt0);
    p.g.rt1 = reinterpret_cast<Item*>(base + kOffRt1);
    p.g.rc0 = reinterpret_cast<Item*>(base + kOffRc0);
    p.g.rc1 = reinterpret_cast<Item*>(base + kOffRc1);
    p.g.tcap = kTcap;
    p.g.ccap = kCcap;
    p.g.n = n;
    p.g.src = src;
    p.te = kTe;
    p.large_deg = kLarge;
    p.chunk = kChunk;
    p.mode = 1;
    p.srcs = reinterpret_cast<const int*>(base + kOffSrc);
    p.nsrc = 1;
    p.max_rounds = 2LL * n + 16;
    p.solo_waves = 2;
    e = launch_update(p, ds->grid, kBlock, s);
    if (e != cudaSuccess) return fail(DSSSP_E_CUDA, "sssp_noalloc: update kernel: %s", cudaGetErrorString(e));
    const unsigned ob = (unsigned)((n + kBlock - 1) / kBlock < 1024 ? (n + kBlock - 1) / kBlock : 1024);
    k_noalloc_out<<<ob, kBlock, 0, s>>>(base, n, d_parent, reinterpret_cast<long long*>(d_dist));
    count_launch(1);
    int status = 0;
    unsigned long long dist_ovf = 0;
    e = cudaMemcpyAsync(&status, base + kOffCtl + offsetof(Ctl, status), sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&dist_ovf, base + kOffCtl + offsetof(Ctl, stat) + sizeof(unsigned long long) * ST_DIST_OVF,
                            sizeof(dist_ovf), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(DSSSP_E_CUDA, "sssp_noalloc: %s", cudaGetErrorString(e));
    if (status == DSSSP_E_INVAL) return fail(DSSSP_E_INVAL, "sssp_noalloc: malformed CSR (offsets, ids or weights)");
    if (status != 0) return fail(status, "sssp_noalloc: device status %d", status);
    if (dist_ovf) return fail(DSSSP_E_OVERFLOW, "sssp_noalloc: a distance does not fit below 2^32-1");
    return DSSSP_OK;
}
