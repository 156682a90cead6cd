// noalloc.cu -- slant-stack Radon for callers that cannot allocate device
// memory.
//
// rg_radon_slantstack needs scratch: the per-view constants of its plan, the
// two line-pair copies of the image and, unless the sinogram is view-major,
// a view-major result buffer.  It takes them from the caller's workspace or
// from the stream-ordered pool, and it caches plans in cudaMalloc'd memory.
// Some callers cannot do any of that: a process that has handed all of its
// device memory to another framework's pool at start-up, or a
// data-acquisition loop that must not allocate once it runs (cudaMalloc and
// cudaFree may synchronise the whole device and stall the streams that move
// detector frames).  For them, rg_radon_slantstack_noalloc keeps all its
// scratch in one file-scope __device__ array of kNoAllocBytes (32 MiB), which
// every GPU that loads the library holds until the process exits.  The call
// runs the same kernels as rg_radon_slantstack and calls no cudaMalloc,
// cudaFree or other allocating routine; the per-view table is built in a
// static host array (under a mutex) and copied into the scratch on the
// caller's stream.
//
// Host code cannot use the array's name as a device address (it names a
// host-side shadow), so the first call on each device, with that device
// current, looks up the device address with cudaGetSymbolAddress and caches
// it together with the identity of the device's current context; that first
// call should come before any stream capture begins on the device.  A call
// that finds another context there (the old one was destroyed, e.g. by
// cudaDeviceReset, and the module loaded again) looks the address up anew.
//
// All calls on a device share the one array, and each call overwrites every
// byte it later reads (the view table, both line-pair copies with their zero
// pads, and the result buffer), so nothing needs clearing between calls.
// Calls whose work overlaps on the GPU (different streams, or host threads
// racing on one device) race on the array: serialise them on one stream.
#include <mutex>

#include "rg_internal.cuh"

namespace rg {
namespace {

constexpr size_t kNoAllocBytes = size_t(32) << 20;
constexpr int kNoAllocMaxViews = 4096;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_mu;

// Per device: the scratch's device address and the id of the context it
// was resolved in.
struct ScratchAddr {
    void *ptr = nullptr;
    unsigned long long ctx_id = 0;
};
ScratchAddr g_addr[kMaxDevices];

// Identity of the calling thread's current context (the device's primary
// context under the runtime API), from the driver through the runtime's
// entry-point query, so the library does not link libcuda itself.
int current_context_id(unsigned long long *id)
{
    typedef int (*GetCurrent)(void **);
    typedef int (*GetId)(void *, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        RG_CK(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                               cudaEnableDefault, &q1));
        RG_CK(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault,
                                               &q2));
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return set_error(RG_EUNSUPPORTED, "driver lacks cuCtxGetCurrent/cuCtxGetId");
        get_current = (GetCurrent)f1;
        get_id = (GetId)f2;
    }
    void *ctx = nullptr;
    *id = 0;
    if (get_current(&ctx) != 0)
        return set_error(RG_ECUDA, "cuCtxGetCurrent failed for the no-alloc scratch");
    if (ctx && get_id(ctx, id) != 0)
        return set_error(RG_ECUDA, "cuCtxGetId failed for the no-alloc scratch");
    return RG_OK;      // *id stays 0 while the thread has no current context
}

// Device address of g_noalloc_scratch on the current device: looked up once
// per device (and again if the device's context was replaced).  Caller holds
// g_mu.
int scratch_address(void **out)
{
    int dev = 0;
    RG_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(RG_EUNSUPPORTED, "device ordinal %d beyond %d", dev, kMaxDevices);
    unsigned long long ctx = 0;
    int rc = current_context_id(&ctx);
    if (rc) return rc;
    ScratchAddr &a = g_addr[dev];
    if (!a.ptr || ctx == 0 || a.ctx_id != ctx) {
        // cudaGetSymbolAddress also makes the device's primary context
        // current when the thread has none yet; read its id after it.
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(no-alloc scratch)");
        if ((rc = current_context_id(&ctx))) return rc;
        a.ptr = p;
        a.ctx_id = ctx;
    }
    *out = a.ptr;
    return RG_OK;
}

// Host staging of the per-view table (guarded by g_mu; a pageable-memory
// cudaMemcpyAsync has consumed its source when it returns).
View g_views[kNoAllocMaxViews];

}  // namespace
}  // namespace rg

using namespace rg;

extern "C" int rg_radon_slantstack_noalloc(rg_image phantom, rg_image radon, void *stream)
{
    RG_TRACE();
    int rc = validate_ss(phantom, radon);
    if (rc) return rc;
    const int N = phantom.lines, R = radon.lines, A = radon.columns;
    if (A > kNoAllocMaxViews)
        return set_error(RG_EINVAL, "no-alloc Radon: %d views exceed the limit of %d", A,
                         kNoAllocMaxViews);
    const bool direct = radon.column_stride == 1 && radon.line_stride == radon.lines;
    const size_t vbytes = Scratch::align(sizeof(View) * A);
    const size_t pbytes = Scratch::align(radon_pairs_bytes(N));
    const size_t obytes = direct ? 0 : Scratch::align((size_t)R * A * sizeof(float));
    const size_t need = vbytes + 2 * pbytes + obytes;
    if (need > kNoAllocBytes)
        return set_error(RG_EINVAL, "no-alloc Radon: %zu bytes of scratch needed for a %d^2 "
                         "image and %d x %d sinogram, the static scratch holds %zu", need, N, R,
                         A, kNoAllocBytes);
    std::lock_guard<std::mutex> lock(g_mu);
    SSPlan p;
    if ((rc = ss_views_compute(p, make_ss_geom(phantom, radon), nullptr, A, g_views))) return rc;
    void *base = nullptr;
    if ((rc = scratch_address(&base))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    char *b = (char *)base;
    p.d_views = (View *)b;
    float2 *prow = (float2 *)(b + vbytes);
    float2 *pcol = (float2 *)(b + vbytes + pbytes);
    float *out_am = (float *)(b + vbytes + 2 * pbytes);
    RG_CK(cudaMemcpyAsync(p.d_views, g_views, sizeof(View) * A, cudaMemcpyHostToDevice, st));
    rc = launch_line_pairs(phantom.data, phantom.column_stride, phantom.line_stride, N, prow,
                           pcol, st);
    if (!rc) rc = launch_radon(p, prow, pcol, direct ? radon.data : out_am, R, nullptr, 0, st);
    if (!rc && !direct)
        rc = launch_from_am(out_am, R, A, radon.data, radon.column_stride, radon.line_stride, st);
    p.d_views = nullptr;   // not owned
    return rc;
}
