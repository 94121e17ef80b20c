// Allocation-free reconstruction of one slice.
//
// Who needs this: callers that must not allocate device memory themselves -- for example a
// plugin running inside a host application that owns a fixed device-memory pool (or a caching
// allocator) and forbids other allocations on the device, or code whose allocation calls would
// synchronise the device at a point where that is not allowed.  They can still hand us the
// sinogram and the output slice as device pointers.
//
// The scratch this path needs (FFT twiddles, filter, row jobs, per-view geometry and the 1/16
// sub-sample tables) lives in one file-scope __device__ array of kNoAllocScratchBytes.  Every GPU
// that loads this library keeps that array for the life of the process.  All calls share it
// and it keeps the previous call's contents; nothing in it has to start at zero, because each
// word a kernel reads is written earlier in the same call.  Two calls whose work overlaps on
// the GPU (different streams, or different host threads on one device) race on the array.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "rv_internal.h"

namespace rv {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;   // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the array, resolved with the device current (host code cannot use the
// symbol's host-side stand-in as a device pointer).  It is resolved on the first call on a device
// and again whenever the device's context has changed since: a device reset
// (CudaReconstResourceFree(ri, true), or the caller's own cudaDeviceReset) destroys the context,
// the module is loaded afresh in the next one, and the array may then sit at another address.
// A cached address from the old context is never handed to a kernel.
constexpr int kMaxDevices = 64;
struct ScratchAddr {
    void* ptr;
    unsigned long long ctx;   // context the address was resolved in (0: unknown, always resolve)
};
static ScratchAddr g_scratch_addr[kMaxDevices] = {};
static std::mutex g_scratch_mu;

static void* scratch_for_current_device(int* code) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        *code = RV_ERR_SET_DEVICE;
        set_error(RV_ERR_SET_DEVICE, "RvReconstructSliceNoAlloc: no usable current device");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    ScratchAddr& a = g_scratch_addr[dev];
    const unsigned long long ctx = current_context_id();
    if (a.ptr && ctx != 0 && a.ctx == ctx) return a.ptr;
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
        a.ptr = nullptr;
        set_error(RV_ERR_LAUNCH, std::string("cudaGetSymbolAddress of the scratch array: ") + cudaGetErrorString(e));
        *code = RV_ERR_LAUNCH;
        return nullptr;
    }
    a.ptr = ptr;
    a.ctx = current_context_id();   // the resolution made the device's context current if it was not
    return ptr;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace rv

using namespace rv;

extern "C" int RvReconstructSliceNoAlloc(const short* d_sino, int nviews, int ixdim, int iInterpolation,
                                         double center, const float* fdeg, float fTiltAngle,
                                         const float* fFilter, int* d_slice, void* stream) {
    if (!d_sino || !fdeg || !fFilter || !d_slice || nviews < 1 || ixdim < 4) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvReconstructSliceNoAlloc: NULL pointer or empty sinogram");
        return RV_ERR_BAD_ARGUMENT;
    }
    const Dims d = make_dims(ixdim, iInterpolation);
    if (d.ndimp > kMaxNdimp || d.ixdimp > kMaxIxdimp) {
        set_error(RV_ERR_UNSUPPORTED, "RvReconstructSliceNoAlloc: ixdim*zoom beyond 16384");
        return RV_ERR_UNSUPPORTED;
    }
    const int pad = ref_table_fmt();
    const long long tstride = ref_table_stride(d.ixdimp, pad);
    // scratch layout: twiddles | filter | row jobs | geometry | tables
    const size_t o_tw = 0;
    const size_t o_filt = align256(o_tw + (size_t)d.ndim * sizeof(float2));   // per-pass twiddle table
    const size_t o_jobs = align256(o_filt + (size_t)d.ndim * sizeof(float));
    const size_t o_geom = align256(o_jobs + (size_t)nviews * sizeof(RowJob));
    const size_t o_tab = align256(o_geom + (size_t)nviews * sizeof(float4));
    const size_t need = o_tab + (size_t)nviews * (size_t)tstride * sizeof(int);
    if (need > kNoAllocScratchBytes) {
        set_error(RV_ERR_UNSUPPORTED,
                  "RvReconstructSliceNoAlloc: views x detector width need " + std::to_string(need) +
                      " bytes of scratch; the fixed scratch array holds " + std::to_string(kNoAllocScratchBytes));
        return RV_ERR_UNSUPPORTED;
    }
    int code = 0;
    unsigned char* base = static_cast<unsigned char*>(scratch_for_current_device(&code));
    if (!base) return code;
    cudaStream_t s = (cudaStream_t)stream;

    std::vector<float2> tw;
    fft_twiddles(d.ndimp, tw);
    std::vector<RowJob> jobs(nviews);
    std::vector<float4> geom(nviews);
    for (int v = 0; v < nviews; v++) {
        RowJob j{};
        j.src_row = v;
        j.dst = v;
        jobs[v] = j;
        float fc, fs, fo;
        view_geometry(d, center, fdeg[v], fTiltAngle, &fc, &fs, &fo);
        geom[v] = make_float4(fc, fs, fo, ray_regime_tag(fc, fs));
    }
    if (!cuda_ok(cudaMemcpyAsync(base + o_tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice, s),
                 RV_ERR_COPY_H2D, "twiddles") ||
        !cuda_ok(cudaMemcpyAsync(base + o_filt, fFilter, (size_t)d.ndim * sizeof(float), cudaMemcpyHostToDevice, s),
                 RV_ERR_COPY_H2D, "filter") ||
        !cuda_ok(cudaMemcpyAsync(base + o_jobs, jobs.data(), jobs.size() * sizeof(RowJob), cudaMemcpyHostToDevice, s),
                 RV_ERR_COPY_H2D, "row jobs") ||
        !cuda_ok(cudaMemcpyAsync(base + o_geom, geom.data(), geom.size() * sizeof(float4), cudaMemcpyHostToDevice, s),
                 RV_ERR_COPY_H2D, "geometry"))
        return RvGetLastError();
    FilterLaunch fl{};
    fl.src = d_sino;
    fl.raw = 0;
    fl.jobs = reinterpret_cast<const RowJob*>(base + o_jobs);
    fl.njobs = nviews;
    fl.filt = reinterpret_cast<const float*>(base + o_filt);
    fl.tw = reinterpret_cast<const float2*>(base + o_tw);
    fl.table = reinterpret_cast<int*>(base + o_tab);
    fl.mode = RV_MODE_REF;
    fl.d = d;
    fl.ic = (int)center;
    fl.table_stride = tstride;
    fl.table_fmt = pad;
    if (!cuda_ok(launch_filter(fl, s), RV_ERR_LAUNCH, "filter kernel")) return RV_ERR_LAUNCH;
    BackprojLaunch bl{};
    bl.table = reinterpret_cast<const int*>(base + o_tab);
    bl.geom = reinterpret_cast<const float4*>(base + o_geom);
    bl.nviews = nviews;
    bl.nslices = 1;
    bl.ixdimp = d.ixdimp;
    bl.table_stride = tstride;
    bl.slice_table_stride = tstride * nviews;
    bl.out = d_slice;
    bl.out_slice_stride = (long long)d.ixdimp * d.ixdimp;
    bl.mode = RV_MODE_REF;
    bl.table_fmt = pad;
    if (!cuda_ok(launch_backproject(bl, s), RV_ERR_LAUNCH, "back-projection kernel")) return RV_ERR_LAUNCH;
    if (!cuda_ok(cudaStreamSynchronize(s), RV_ERR_LAUNCH, "no-alloc slice")) return RV_ERR_LAUNCH;
    if (const unsigned ks = take_kernel_status(s)) {
        set_error(RV_ERR_KERNEL_STATUS, std::string("back-projection: ") + kernel_status_text(ks));
        return RV_ERR_KERNEL_STATUS;
    }
    return 0;
}

// The address RvReconstructSliceNoAlloc would hand its kernels on the current device now
// (*resolved, by the same context-checked cache) and a fresh cudaGetSymbolAddress of the array
// (*fresh).  Host-only: nothing is launched, copied or allocated.  Tests use it to show that a
// device reset never leaves the entry point with an address from the destroyed context.
extern "C" int RvNoAllocScratchAddress(void** resolved, void** fresh) {
    if (!resolved || !fresh) return RV_ERR_BAD_ARGUMENT;
    int code = 0;
    *resolved = scratch_for_current_device(&code);
    if (!*resolved) return code;
    *fresh = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(fresh, g_noalloc_scratch), RV_ERR_LAUNCH, "cudaGetSymbolAddress"))
        return RV_ERR_LAUNCH;
    return 0;
}
