// Host side of the drop-in: RecView's CUDA entry points (source/cudaReconst.h) implemented on the
// library's kernels, plus error reporting, geometry and the device queries.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "rv_internal.h"

// The application (RecView) defines the progress/abort hook; a library user without it may
// register one with RvSetProgressCallback.
extern "C" bool DBProjDlgCtrl(RECONST_INFO* ri, int iProgStep, int iSino, int* pCurrStep)
    __attribute__((weak));

namespace rv {

// ---------------------------------------------------------------------------- errors ---------
static RvErrorCallback g_err_cb = nullptr;
static RvProgressCallback g_progress_cb = nullptr;
static thread_local int t_last_code = 0;
static thread_local std::string t_last_msg;

void set_error(int code, const std::string& msg) {
    t_last_code = code;
    t_last_msg = msg;
    RvErrorCallback cb = g_err_cb;
    if (cb) cb(code, t_last_msg.c_str());
}

static bool progress(RECONST_INFO* ri, int step, int i, int* cur) {
    if (DBProjDlgCtrl) return DBProjDlgCtrl(ri, step, i, cur);
    if (g_progress_cb) return g_progress_cb(ri, step, i, cur);
    return false;
}

// ---------------------------------------------------------------------------- contexts -------
// The driver's cuCtxGetCurrent / cuCtxGetId, looked up through the runtime so the library needs
// no link-time dependency on libcuda (it still loads on machines without a driver).
typedef int (*PfnCtxGetCurrent)(void** ctx);
typedef int (*PfnCtxGetId)(void* ctx, unsigned long long* id);

unsigned long long current_context_id() {
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(f);
    });
    if (!get_current || !get_id) return 0;
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return 0;
    unsigned long long id = 0;
    if (get_id(ctx, &id) != 0) return 0;   // e.g. the context was destroyed by a reset
    return id;
}

// ---------------------------------------------------------------------------- geometry -------
Dims make_dims(int ixdim, int iInterpolation) {
    // source/general.cpp:2021-2035 (same double log / pow arithmetic)
    Dims d;
    d.ixdim = ixdim;
    d.iZooming = (iInterpolation > RV_ZOOMING_NONE) ? (iInterpolation - RV_ZOOMING_NONE) : 0;
    d.iIntpDim = (int)pow(2.0, d.iZooming);
    d.ndimp = (int)(log((double)ixdim) / 0.69314718055994530941723212145818) + 1 + d.iZooming;
    d.ndim = (int)pow(2.0, d.ndimp);
    d.ixdimp = ixdim * d.iIntpDim;
    d.ixdimh = d.ixdimp / 2;
    d.ihoffset = d.ndim / 2 - 1 - d.ixdimh;
    return d;
}

// This translation unit is compiled with -ffp-contract=off: each float operation below is
// rounded separately, as in the reference's x64 build.
float fcenter_of(const Dims& d, double center) {
    // source/general.cpp:2036-2037 ((int)center truncates the double centre)
    const int ic = (int)center;
    if (d.iIntpDim == 1) {
        float a = (float)d.ixdimh + (float)center;
        a = a - (float)ic;
        return a * (float)RV_DBPT_GINTP;
    }
    float fr = (float)center - (float)ic;
    fr = fr * (float)d.iIntpDim;
    fr = (float)d.ixdimh + fr;
    return fr * (float)RV_DBPT_GINTP;
}

void view_geometry(const Dims& d, double center, float fdeg, float tilt, float* fcos, float* fsin,
                   float* foffset) {
    // source/general.cpp:2139-2142; DEG_TO_RAD = 0.0174532925199 (source/constants.h:3)
    const float deg = fdeg + tilt;
    const double th = (double)deg * 0.0174532925199;
    const float c = (float)(cos(th) * RV_DBPT_GINTP);
    const float s = (float)(-sin(th) * RV_DBPT_GINTP);
    const float sum = c + s;
    const float prod = (float)d.ixdimh * sum;
    *fcos = c;
    *fsin = s;
    *foffset = fcenter_of(d, center) - prod;
}

void fft_twiddles(int np, std::vector<float2>& out) {
    // CFft::Init1(np, -1) (source/cfft.cpp:374-410): angle a = -(float)2pi * (i/n) in float;
    // cos/sin taken correctly rounded (the double result rounded to float).  Stored per radix-2
    // pass: pass l (2^l butterflies per group) reads w[q << (np-1-l)], q < 2^l, from
    // out[2^l + q], so a warp's twiddle reads are consecutive addresses in every pass.
    const int n = 1 << np, half = n / 2;
    std::vector<float2> w(half);
    float p0 = (float)6.283185307178;
    p0 = p0 * -1.0f;
    for (int i = 0; i < half; i++) {
        const float a = p0 * ((float)i / (float)n);
        w[i] = make_float2((float)cos((double)a), (float)sin((double)a));
    }
    out.assign(n, make_float2(1.0f, 0.0f));
    for (int l = 1; l < np; l++)
        for (int q = 0; q < (1 << l); q++) out[(1 << l) + q] = w[(size_t)q << (np - 1 - l)];
}

// ---------------------------------------------------------------------------- context -------
// Device buffers cached across calls for one RECONST_INFO (the reference caches d_ifp/d_igp/
// d_px/d_strip in the struct itself; source/cudaReconstHost.cpp:19-141).
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    bool ensure(size_t need) {
        if (need <= bytes && p) return true;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (cudaMalloc(&p, need ? need : 16) != cudaSuccess) return false;
        bytes = need;
        return true;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
};

struct RiContext {
    int device = -1;
    DevBuf out, table, rows, jobs, geom, filt, tw, raw, sino_out, shift, rowptr;
    void* h_stage = nullptr;   // pinned staging for row gathers
    size_t h_stage_bytes = 0;
    int tw_np = -1;
    // filtered views kept for RQFLAGS_SINOGRAMKEPT (source/cudaReconstHost.cpp:658)
    bool kept = false;
    int kept_ixdim = 0, kept_interp = 0, kept_start = 0, kept_step = 0, kept_mult = 0, kept_off = 0;
    int kept_fmt = 0;
    std::vector<int> kept_views;

    bool stage(size_t need) {
        if (need <= h_stage_bytes && h_stage) return true;
        if (h_stage) cudaFreeHost(h_stage);
        h_stage = nullptr;
        h_stage_bytes = 0;
        if (cudaMallocHost(&h_stage, need ? need : 16) != cudaSuccess) return false;
        h_stage_bytes = need;
        return true;
    }
    void release() {
        DevBuf* all[] = {&out, &table, &rows, &jobs, &geom, &filt, &tw, &raw, &sino_out, &shift, &rowptr};
        for (DevBuf* b : all) b->release();
        if (h_stage) cudaFreeHost(h_stage);
        h_stage = nullptr;
        h_stage_bytes = 0;
        tw_np = -1;
        kept = false;
        kept_views.clear();
    }
};

static RiContext* ctx_of(RECONST_INFO* ri, bool create) {
    if (ri->d_p && ri->max_d_p == RV_CTX_TAG) return reinterpret_cast<RiContext*>(ri->d_p);
    if (!create) return nullptr;
    RiContext* c = new RiContext();
    ri->d_p = reinterpret_cast<RvFloat2*>(c);
    ri->max_d_p = RV_CTX_TAG;
    return c;
}

static void publish_fields(RECONST_INFO* ri, RiContext* c) {
    // keep the reference's cache fields meaningful for callers that inspect them
    ri->d_ifp = static_cast<int*>(c->out.p);
    ri->max_d_ifp = (unsigned)(c->out.bytes > 0xffffffffu ? 0xffffffffu : c->out.bytes);
    ri->d_igp = static_cast<int*>(c->table.p);
    ri->max_d_igp = (unsigned)(c->table.bytes > 0xffffffffu ? 0xffffffffu : c->table.bytes);
    ri->d_strip = static_cast<short*>(c->rows.p);
    ri->max_d_strip = (unsigned)(c->rows.bytes > 0xffffffffu ? 0xffffffffu : c->rows.bytes);
}

static bool upload_twiddles(RiContext* c, int np, cudaStream_t s) {
    if (c->tw_np == np && c->tw.p) return true;
    std::vector<float2> tw;
    fft_twiddles(np, tw);
    if (!c->tw.ensure(tw.size() * sizeof(float2))) {
        set_error(RV_ERR_DEVICE_OOM, "twiddle buffer");
        return false;
    }
    if (!cuda_ok(cudaMemcpyAsync(c->tw.p, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice, s),
                 RV_ERR_COPY_H2D, "twiddles"))
        return false;
    if (!cuda_ok(cudaStreamSynchronize(s), RV_ERR_COPY_H2D, "twiddles")) return false;
    c->tw_np = np;
    return true;
}

static void fail(RECONST_INFO* ri, int code, const std::string& msg) {
    set_error(code, msg);
    ri->iStatus = RECONST_INFO_ERROR;
}

}  // namespace rv

using namespace rv;

// ============================================================================ drop-in ==========
extern "C" void CudaReconstHost(RECONST_INFO* ri, int idev, bool bReport, bool bEnStream) {
    if (!ri) {
        set_error(RV_ERR_BAD_ARGUMENT, "CudaReconstHost: ri is NULL");
        return;
    }
    if (cudaSetDevice(idev) != cudaSuccess) {
        fail(ri, RV_ERR_SET_DEVICE, "cudaSetDevice error");
        return;
    }
    const Dims d = make_dims(ri->ixdim, ri->iInterpolation);
    if (ri->ixdim < 4 || !ri->iSinogr || !ri->fFilter || !ri->fdeg || !ri->bInc || !ri->iReconst ||
        !ri->nSinogr || ri->iStepSino < 1 || ri->iStartSino < 0 || ri->iMultiplex < 1) {
        fail(ri, RV_ERR_BAD_ARGUMENT, "CudaReconstHost: inconsistent RECONST_INFO");
        return;
    }
    if (d.ndimp > kMaxNdimp || d.ixdimp > kMaxIxdimp) {
        fail(ri, RV_ERR_UNSUPPORTED, "CudaReconstHost: ixdim*zoom beyond 16384 / FFT beyond 16384");
        return;
    }
    RiContext* c = ctx_of(ri, true);
    c->device = idev;
    cudaStream_t s = 0;
    if (bEnStream) {
        // two cached streams as the reference keeps (source/cudaReconstHost.cpp:685-703); this
        // implementation issues the whole slice on stream1.
        cudaError_t e1 = cudaSuccess, e2 = cudaSuccess;
        if (!ri->stream1) e1 = cudaStreamCreate(reinterpret_cast<cudaStream_t*>(&ri->stream1));
        if (!ri->stream2) e2 = cudaStreamCreate(reinterpret_cast<cudaStream_t*>(&ri->stream2));
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            if (e1 == cudaSuccess && ri->stream1) cudaStreamDestroy((cudaStream_t)ri->stream1);
            if (e2 == cudaSuccess && ri->stream2) cudaStreamDestroy((cudaStream_t)ri->stream2);
            ri->stream1 = ri->stream2 = nullptr;
            set_error(RV_ERR_STREAM, "cudaStreamCreate failed; using the default stream");
        } else {
            s = (cudaStream_t)ri->stream1;
        }
    }
    const int ixdimp = d.ixdimp;
    const int intcenter = (int)ri->center;
    // ---- views (source/cudaReconstHost.cpp:712-738) -----------------------------------------
    std::vector<int> views, sidxs;
    const int iProgStep = ri->iLenSinogr / 20;
    int iCurrStep = 0;
    for (int i = ri->iStartSino; i < ri->iLenSinogr - 1; i += ri->iStepSino) {
        const int isino = (i - ri->iStartSino) / ri->iStepSino;
        if (bReport && (isino % 20 == 0)) {
            if (progress(ri, iProgStep, i, &iCurrStep)) break;
        }
        if (!(ri->bInc[i] & RV_BINC_SAMPLE)) continue;
        const int sidx = i * ri->iMultiplex + ri->iOffset;
        if (sidx >= ri->maxSinogrLen) break;
        if (ri->dReconFlags & (RV_RQFLAGS_USEONLYEVENFRAMES | RV_RQFLAGS_USEONLYODDFRAMES)) {
            if (i & 1) {
                if (ri->dReconFlags & RV_RQFLAGS_USEONLYEVENFRAMES) continue;
            } else {
                if (ri->dReconFlags & RV_RQFLAGS_USEONLYODDFRAMES) continue;
            }
        }
        (*(ri->nSinogr))++;
        views.push_back(i);
        sidxs.push_back(sidx);
    }
    const int nv = (int)views.size();
    // ---- R10: reuse of kept filtered views (source/cudaReconstHost.cpp:658,775) -------------
    bool bDeconv = !(ri->dReconFlags & RV_RQFLAGS_SINOGRAMKEPT) || !c->kept || d.iIntpDim != 1 ||
                   c->kept_ixdim != ri->ixdim || c->kept_interp != ri->iInterpolation ||
                   c->kept_start != ri->iStartSino || c->kept_step != ri->iStepSino ||
                   c->kept_mult != ri->iMultiplex || c->kept_off != ri->iOffset || c->kept_views != views ||
                   c->kept_fmt != ref_table_fmt();
    const int tfmt = ref_table_fmt();
    const size_t table_stride = (size_t)ref_table_stride(ixdimp, tfmt);
    if (!c->out.ensure((size_t)ixdimp * ixdimp * sizeof(int))) {
        fail(ri, RV_ERR_DEVICE_OOM, "Out of CUDA device memory (slice)");
        return;
    }
    if (bDeconv && nv > 0) {
        ri->iSinoCenter = intcenter;
        c->kept = false;
        const size_t row_bytes = (size_t)ri->ixdim * sizeof(short);
        if (!c->table.ensure((size_t)nv * table_stride * sizeof(int)) || !c->rows.ensure(nv * row_bytes) ||
            !c->jobs.ensure(nv * sizeof(RowJob)) || !c->filt.ensure((size_t)d.ndim * sizeof(float))) {
            fail(ri, RV_ERR_DEVICE_OOM, "Out of CUDA device memory (filtered views)");
            return;
        }
        // where the device reads pageable host memory directly (shared page tables), the filter
        // takes each view's row from the caller's row pointer; otherwise the rows are gathered
        // into pinned staging and copied
        const bool direct = host_direct_access();
        const size_t gather_bytes = direct ? (size_t)nv * sizeof(short*) : (size_t)nv * row_bytes;
        if (!c->stage(gather_bytes + nv * sizeof(RowJob)) || (direct && !c->rowptr.ensure(gather_bytes))) {
            fail(ri, direct ? RV_ERR_DEVICE_OOM : RV_ERR_PINNED_ALLOC, "row staging");
            return;
        }
        char* hs = static_cast<char*>(c->h_stage);
        if (direct) {
            const short** hp = reinterpret_cast<const short**>(hs);
            for (int v = 0; v < nv; v++) hp[v] = ri->iSinogr[sidxs[v]];
        } else {
            for (int v = 0; v < nv; v++) memcpy(hs + v * row_bytes, ri->iSinogr[sidxs[v]], row_bytes);
        }
        RowJob* hj = reinterpret_cast<RowJob*>(hs + gather_bytes);
        for (int v = 0; v < nv; v++) {
            RowJob j{};
            j.src_row = v;
            j.dst = v;
            hj[v] = j;
        }
        if (!upload_twiddles(c, d.ndimp, s)) { ri->iStatus = RECONST_INFO_ERROR; return; }
        if (!cuda_ok(cudaMemcpyAsync(direct ? c->rowptr.p : c->rows.p, hs, gather_bytes, cudaMemcpyHostToDevice, s),
                     RV_ERR_COPY_H2D, "sinogram rows") ||
            !cuda_ok(cudaMemcpyAsync(c->jobs.p, hj, nv * sizeof(RowJob), cudaMemcpyHostToDevice, s), RV_ERR_COPY_H2D,
                     "row jobs") ||
            !cuda_ok(cudaMemcpyAsync(c->filt.p, ri->fFilter, (size_t)d.ndim * sizeof(float), cudaMemcpyHostToDevice, s),
                     RV_ERR_COPY_H2D, "filter")) {
            ri->iStatus = RECONST_INFO_ERROR;
            return;
        }
        FilterLaunch fl{};
        fl.src = c->rows.p;
        fl.row_ptr = direct ? static_cast<const short* const*>(c->rowptr.p) : nullptr;
        fl.raw = 0;
        fl.jobs = static_cast<const RowJob*>(c->jobs.p);
        fl.njobs = nv;
        fl.filt = static_cast<const float*>(c->filt.p);
        fl.tw = static_cast<const float2*>(c->tw.p);
        fl.table = static_cast<int*>(c->table.p);
        fl.mode = RV_MODE_REF;
        fl.d = d;
        fl.ic = intcenter;
        fl.table_stride = (long long)table_stride;
        fl.table_fmt = tfmt;
        if (!cuda_ok(launch_filter(fl, s), RV_ERR_LAUNCH, "filter kernel")) {
            ri->iStatus = RECONST_INFO_ERROR;
            return;
        }
        c->kept = true;
        c->kept_ixdim = ri->ixdim;
        c->kept_interp = ri->iInterpolation;
        c->kept_start = ri->iStartSino;
        c->kept_step = ri->iStepSino;
        c->kept_mult = ri->iMultiplex;
        c->kept_off = ri->iOffset;
        c->kept_views = views;
        c->kept_fmt = tfmt;
    }
    // ---- geometry + back-projection ---------------------------------------------------------
    if (nv > 0) {
        const int shift16 = bDeconv ? 0 : RV_DBPT_GINTP * (intcenter - ri->iSinoCenter);
        std::vector<float4> geom(nv);
        for (int v = 0; v < nv; v++) {
            float fc, fs, fo;
            view_geometry(d, ri->center, ri->fdeg[views[v]], ri->fTiltAngle, &fc, &fs, &fo);
            if (shift16) fo = fo + (float)shift16;  // source/cudaReconst.cu:222
            geom[v] = make_float4(fc, fs, fo, ray_regime_tag(fc, fs));
        }
        if (!c->geom.ensure(nv * sizeof(float4))) {
            fail(ri, RV_ERR_DEVICE_OOM, "geometry table");
            return;
        }
        if (!cuda_ok(cudaMemcpyAsync(c->geom.p, geom.data(), nv * sizeof(float4), cudaMemcpyHostToDevice, s),
                     RV_ERR_COPY_H2D, "geometry")) {
            ri->iStatus = RECONST_INFO_ERROR;
            return;
        }
        BackprojLaunch bl{};
        bl.table = static_cast<const int*>(c->table.p);
        bl.geom = static_cast<const float4*>(c->geom.p);
        bl.nviews = nv;
        bl.nslices = 1;
        bl.ixdimp = ixdimp;
        bl.table_stride = (long long)table_stride;
        bl.slice_table_stride = (long long)table_stride * nv;
        bl.out = c->out.p;
        bl.out_slice_stride = (long long)ixdimp * ixdimp;
        bl.mode = RV_MODE_REF;
        bl.table_fmt = tfmt;
        if (!cuda_ok(launch_backproject(bl, s), RV_ERR_LAUNCH, "back-projection kernel")) {
            ri->iStatus = RECONST_INFO_ERROR;
            return;
        }
    } else {
        if (!cuda_ok(cudaMemsetAsync(c->out.p, 0, (size_t)ixdimp * ixdimp * sizeof(int), s), RV_ERR_MEMSET,
                     "slice memset")) {
            ri->iStatus = RECONST_INFO_ERROR;
            return;
        }
    }
    // ---- copy the slice back (source/cudaReconstHost.cpp:811): by a kernel that writes the
    // caller's buffer directly where the device can, else a device-to-host copy -------------------
    const size_t out_bytes = (size_t)ixdimp * ixdimp * sizeof(int);
    const bool direct_out = host_direct_access() && !(out_bytes & 15) && !(reinterpret_cast<uintptr_t>(ri->iReconst) & 15);
    if (!cuda_ok(direct_out ? launch_copy16(ri->iReconst, c->out.p, out_bytes, s)
                            : cudaMemcpyAsync(ri->iReconst, c->out.p, out_bytes, cudaMemcpyDeviceToHost, s),
                 RV_ERR_COPY_D2H, "slice copy") ||
        !cuda_ok(cudaStreamSynchronize(s), RV_ERR_LAUNCH, "slice")) {
        ri->iStatus = RECONST_INFO_ERROR;
        return;
    }
    if (const unsigned ks = take_kernel_status(s)) {
        fail(ri, RV_ERR_KERNEL_STATUS, std::string("back-projection: ") + kernel_status_text(ks));
        return;
    }
    publish_fields(ri, c);
}

extern "C" void CudaReconstHostFFT(RECONST_INFO* ri, int idev, bool bReport) {
    CudaReconstHost(ri, idev, bReport, false);
}

extern "C" void CudaReconstMemFree(RECONST_INFO* ri) {
    if (!ri) return;
    RiContext* c = ctx_of(ri, false);
    if (c) {
        if (c->device >= 0) cudaSetDevice(c->device);
        c->release();
        delete c;
        ri->d_p = nullptr;
        ri->max_d_p = 0;
    }
    ri->d_ifp = nullptr;
    ri->max_d_ifp = 0;
    ri->d_igp = nullptr;
    ri->max_d_igp = 0;
    ri->d_strip = nullptr;
    ri->max_d_strip = 0;
}

extern "C" void CudaReconstResourceFree(RECONST_INFO* ri, bool bCudaDeviceReset) {
    if (!ri) return;
    cudaSetDevice(ri->iStartSino);
    if (ri->stream1) { cudaStreamDestroy((cudaStream_t)ri->stream1); ri->stream1 = nullptr; }
    if (ri->stream2) { cudaStreamDestroy((cudaStream_t)ri->stream2); ri->stream2 = nullptr; }
    CudaReconstMemFree(ri);
    if (bCudaDeviceReset) {
        cudaDeviceSynchronize();
        cudaDeviceReset();  // ends this process's context only
    }
}

// ---- R1 on the device: GenerateSinogramThread semantics (source/general.cpp:2377-2532) -------
extern "C" void CudaSinogramHost(RECONST_INFO* ri, int idev, bool bReport) {
    (void)bReport;
    if (!ri) {
        set_error(RV_ERR_BAD_ARGUMENT, "CudaSinogramHost: ri is NULL");
        return;
    }
    if (cudaSetDevice(idev) != cudaSuccess) {
        fail(ri, RV_ERR_SET_DEVICE, "cudaSetDevice error");
        return;
    }
    const int isino = ri->maxSinogrLen;
    const int W = ri->ixdim, mult = ri->iMultiplex;
    if (W < 1 || mult < 1 || isino < 2 || !ri->iSinogr || !ri->bInc || !ri->fexp || !ri->fdeg || ri->iStepSino < 1) {
        fail(ri, RV_ERR_BAD_ARGUMENT, "CudaSinogramHost: inconsistent RECONST_INFO");
        return;
    }
    const int ibin = (ri->iInterpolation == 0) ? 4 : ((ri->iInterpolation == 1) ? 2 : 1);
    const int pixmin = (ri->iFlag & RV_READTIF8bit) ? RV_SINOGRAM_PIXEL_MIN8bit : RV_SINOGRAM_PIXEL_MIN16bit;
    const char* bInc = ri->bInc;
    std::vector<RowJob> jobs;
    std::vector<int> shifts;
    bool error = false;
    int i0 = -1, i1 = -1;
    for (int i = 0; i < isino - 1; i++) {
        if (bInc[i] & RV_BINC_NOUSE) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; break; }
    }
    for (int i = 0; i < isino - 1; i++) {
        if ((bInc[i] & RV_BINC_NOUSE) && !(bInc[i] & RV_BINC_SAMPLE)) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; i1 = -1; continue; }
        if (i1 < 0) {
            for (int j = i; j < isino - 1; j++) {
                if (bInc[j] & RV_BINC_SAMPLE) continue;
                i1 = j;
                break;
            }
            if (i1 < 0) {
                if (i0 >= 0) i1 = i0;
                else { error = true; break; }
            }
        }
        if (i0 < 0 || i1 < 0) { error = true; break; }
        if (i % ri->iStepSino != ri->iStartSino) continue;
        float t0 = ri->fexp[i0];
        const float t1 = ri->fexp[i1];
        const float ti = ri->fexp[i];
        if (t0 == t1) t0 = 0;
        else t0 = (ti - t0) / (t1 - t0);
        const double cth = cos(ri->fdeg[i] * 0.0174532925199), sth = sin(ri->fdeg[i] * 0.0174532925199);
        int idrift = 0;
        bool zero = false;
        if ((ri->drEnd > ri->drStart) && (ri->dReconFlags & RV_RQFLAGS_DRIFTPARAMS)) {
            if ((ri->drStart < i) && (i < ri->drEnd) && ri->drOmit) zero = true;
            const double dd = ri->drX * cth - ri->drY * sth;
            if (i >= ri->drEnd) idrift = (int)dd;
            else if (i > ri->drStart) idrift = (int)(dd * (i - ri->drStart) / (ri->drEnd - ri->drStart));
        }
        if (bInc[i] & RV_BINC_SKIP) zero = true;
        if (!zero && (ri->dReconFlags & RV_RQFLAGS_DRIFTLIST) && ri->piDrift) idrift -= ri->piDrift[i];
        for (int k = 0; k < mult; k++) {
            RowJob j{};
            j.src_row = mult * i + k;
            j.flat0_row = mult * i0 + k;
            j.flat1_row = mult * i1 + k;
            j.dark_row = mult * (isino - 1) + k;
            j.t0 = t0;
            j.dst = mult * i + k;
            j.zero = zero ? 1 : 0;
            jobs.push_back(j);
            shifts.push_back(zero ? 0 : idrift / ibin);
        }
    }
    const int nj = (int)jobs.size();
    if (nj > 0) {
        RiContext* c = ctx_of(ri, true);
        c->device = idev;
        const size_t nrows = (size_t)isino * mult, row_bytes = (size_t)W * sizeof(short);
        if (!c->raw.ensure(nrows * row_bytes) || !c->sino_out.ensure(nrows * row_bytes) ||
            !c->jobs.ensure(nj * sizeof(RowJob)) || !c->shift.ensure(nj * sizeof(int))) {
            fail(ri, RV_ERR_DEVICE_OOM, "Out of CUDA device memory (sinogram)");
            return;
        }
        // where the device reads and writes pageable host memory directly, the kernel works on
        // the caller's rows in place through a table of their pointers; otherwise every row is
        // staged in and the sample rows copied back
        const bool direct = host_direct_access();
        const size_t stage_bytes = direct ? nrows * sizeof(short*) : nrows * row_bytes;
        if (!c->stage(stage_bytes) || (direct && !c->rowptr.ensure(stage_bytes))) {
            fail(ri, direct ? RV_ERR_DEVICE_OOM : RV_ERR_PINNED_ALLOC, "row staging");
            return;
        }
        char* hs = static_cast<char*>(c->h_stage);
        if (direct) {
            short** hp = reinterpret_cast<short**>(hs);
            for (size_t r = 0; r < nrows; r++) hp[r] = ri->iSinogr[r];
        } else {
            for (size_t r = 0; r < nrows; r++) memcpy(hs + r * row_bytes, ri->iSinogr[r], row_bytes);
        }
        cudaStream_t s = 0;
        bool ok = cuda_ok(cudaMemcpyAsync(direct ? c->rowptr.p : c->raw.p, hs, stage_bytes, cudaMemcpyHostToDevice, s),
                          RV_ERR_COPY_H2D, "raw rows") &&
                  cuda_ok(cudaMemcpyAsync(c->jobs.p, jobs.data(), nj * sizeof(RowJob), cudaMemcpyHostToDevice, s), RV_ERR_COPY_H2D, "jobs") &&
                  cuda_ok(cudaMemcpyAsync(c->shift.p, shifts.data(), nj * sizeof(int), cudaMemcpyHostToDevice, s), RV_ERR_COPY_H2D, "shifts");
        if (ok) {
            NormLaunch nl{};
            nl.raw = static_cast<const uint16_t*>(c->raw.p);
            nl.out = static_cast<short*>(c->sino_out.p);
            nl.row_ptr = direct ? static_cast<const uint16_t* const*>(c->rowptr.p) : nullptr;
            nl.jobs = static_cast<const RowJob*>(c->jobs.p);
            nl.njobs = nj;
            nl.ixdim = W;
            nl.pixmin = pixmin;
            nl.zernike = (ri->dReconFlags & RV_RQFLAGS_ZERNIKE) ? 1 : 0;
            nl.shift = static_cast<const int*>(c->shift.p);
            ok = cuda_ok(launch_normalise(nl, s), RV_ERR_LAUNCH, "normalise kernel");
            if (ok && !direct)
                ok = cuda_ok(cudaMemcpyAsync(hs, c->sino_out.p, nrows * row_bytes, cudaMemcpyDeviceToHost, s), RV_ERR_COPY_D2H,
                             "rows");
            if (ok) ok = cuda_ok(cudaStreamSynchronize(s), RV_ERR_LAUNCH, "normalise");
        }
        if (!ok) {
            ri->iStatus = RECONST_INFO_ERROR;
            return;
        }
        if (!direct)
            for (int q = 0; q < nj; q++) memcpy(ri->iSinogr[jobs[q].dst], hs + (size_t)jobs[q].dst * row_bytes, row_bytes);
    }
    if (error) {
        fail(ri, RV_ERR_BAD_ARGUMENT, "CudaSinogramHost: no flat frame brackets a sample frame");
        return;
    }
    ri->iStatus = RECONST_INFO_IDLE;
}

// ---- device queries (source/cudaReconst.cu:449-538) -------------------------------------------
extern "C" int GetCudaDeviceCount(int iMinComputeCapability) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e == cudaErrorNoDevice) return 0;
    if (e == cudaErrorInsufficientDriver) return CUDA_ERROR_INSUFFICIENT_DRIVER;
    if (e != cudaSuccess) return CUDA_ERROR_DEVICE_GETCOUNT;
    for (int i = 0; i < n; i++) {
        cudaDeviceProp pr;
        if (cudaGetDeviceProperties(&pr, i) != cudaSuccess) return i | CUDA_ERROR_DEVICE_GETPROPERTY;
        if (pr.major == 9999 && pr.minor == 9999) return i | CUDA_ERROR_VIRTUAL_DEVICE_DETECTED;
        if (pr.major * 100 + pr.minor * 10 < iMinComputeCapability) return i | CUDA_ERROR_INSUFFICIENT_COMPUTE_CAPABILITY;
    }
    return n;
}

extern "C" int GetCudaMaxThreadsPerBlock(int iDevice) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxThreadsPerBlock, iDevice) != cudaSuccess) return CUDA_ERROR_DEVICE_GETPROPERTY;
    return v;
}

extern "C" int GetCudaWarpSize(int iDevice) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrWarpSize, iDevice) != cudaSuccess) return CUDA_ERROR_DEVICE_GETPROPERTY;
    return v;
}

extern "C" int GetCudaDeviceName(int iDevice, char* pcName, int iszcName) {
    cudaDeviceProp pr;
    if (cudaGetDeviceProperties(&pr, iDevice) != cudaSuccess) return CUDA_ERROR_DEVICE_GETPROPERTY;
    if (pr.major == 9999 && pr.minor == 9999) return CUDA_ERROR_VIRTUAL_DEVICE_DETECTED;
    const int isz = iszcName < 256 ? iszcName : 256;
    for (int i = 0; i < isz; i++) {
        pcName[i] = pr.name[i];
        if (pr.name[i] == 0) break;
    }
    return 0;
}

extern "C" int GetCudaDeviceComputingCapability(int iDevice, int* piMajor, int* piMinor) {
    int ma = 0, mi = 0;
    if (cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, iDevice) != cudaSuccess ||
        cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, iDevice) != cudaSuccess)
        return CUDA_ERROR_DEVICE_GETPROPERTY;
    if (ma == 9999 && mi == 9999) return CUDA_ERROR_VIRTUAL_DEVICE_DETECTED;
    if (piMajor) *piMajor = ma;
    if (piMinor) *piMinor = mi;
    return 0;
}

extern "C" int GetCudaNumberOfCores(int iDevice, int* piCores, int* piProcessors) {
    int ma = 0, sms = 0;
    if (cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, iDevice) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, iDevice) != cudaSuccess)
        return CUDA_ERROR_DEVICE_GETPROPERTY;
    // FP32 lanes per SM: 128 on every architecture this library targets (sm_100 family).
    if (piCores) *piCores = 128;
    if (piProcessors) *piProcessors = sms;
    return 0;
}

extern "C" int GetCudaClockRate(int iDevice, int* piClockRate, int* piMemRate) {
    int clk = 0, mem = 0;
    if (cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, iDevice) != cudaSuccess) return CUDA_ERROR_DEVICE_GETPROPERTY;
    cudaDeviceGetAttribute(&mem, cudaDevAttrMemoryClockRate, iDevice);
    if (piClockRate) *piClockRate = clk;
    if (piMemRate) *piMemRate = mem;
    return 0;
}

extern "C" int CUDA_MALLOC_HOST_INT(int** ptr, size_t size) { return (int)cudaMallocHost((void**)ptr, size); }
extern "C" int CUDA_FREE_HOST(void* ptr) { return (int)cudaFreeHost(ptr); }

// ---- 3-D stitching: out of scope, symbols kept (source/cudaReconstDummy.cpp:27-39) ------------
extern "C" void CudaLsqfitMemAlloc(short**, short**, int*, int*, short**, short**, int, int, int, unsigned long long**) {
    set_error(RV_ERR_UNSUPPORTED, "CudaLsqfitMemAlloc: 3-D stitching is not provided by this library");
}
extern "C" void CudaLsqfitMemFree(short**, short**, int, int, unsigned long long*) {
    set_error(RV_ERR_UNSUPPORTED, "CudaLsqfitMemFree: 3-D stitching is not provided by this library");
}
extern "C" void CudaLsqfitHost(short*, short*, int, int, int, int, int, int, unsigned long long*, unsigned long long*,
                               unsigned long long*, unsigned long long*) {
    set_error(RV_ERR_UNSUPPORTED, "CudaLsqfitHost: 3-D stitching is not provided by this library");
}

// ---- library additions ---------------------------------------------------------------------
extern "C" void RvSetErrorCallback(RvErrorCallback cb) { g_err_cb = cb; }
extern "C" int RvGetLastError(void) { return t_last_code; }
extern "C" const char* RvGetLastErrorMessage(void) { return t_last_msg.c_str(); }
extern "C" void RvClearLastError(void) {
    t_last_code = 0;
    t_last_msg.clear();
}
extern "C" void RvSetProgressCallback(RvProgressCallback cb) { g_progress_cb = cb; }

extern "C" int RvGetDims(int ixdim, int iInterpolation, RvDims* out) {
    if (!out || ixdim < 1) return RV_ERR_BAD_ARGUMENT;
    const Dims d = make_dims(ixdim, iInterpolation);
    out->ixdim = d.ixdim;
    out->iZooming = d.iZooming;
    out->iIntpDim = d.iIntpDim;
    out->ndimp = d.ndimp;
    out->ndim = d.ndim;
    out->ixdimp = d.ixdimp;
    out->ixdimh = d.ixdimh;
    out->ihoffset = d.ihoffset;
    return 0;
}

extern "C" int RvSetFilter(int kind, double cutoff, double order_d, int ndim, float* F) {
    // CGazoDoc::SetFilter (source/gazoDoc.cpp:3762-3811) in float, plus RV_FILT_SHEPP
    // (Shepp-Logan window sinc(pi f / 2), this library's addition, same one-sided layout).
    if (!F || ndim <= 0) return RV_ERR_BAD_ARGUMENT;
    const double PI = 3.1415926535897;  // source/constants.h:4
    const int ndimh = (int)(ndim * cutoff);
    const float order = (float)order_d;
    const float revndim = 1.f / (float)ndim;
    switch (kind) {
    case RV_FILT_HAN:
        for (int i = 0; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const float w = (float)(1 + cos(PI * (double)frac));
            F[i] = ((0.5f * revndim) * (float)i) * w;
        }
        for (int i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_HAM:
        for (int i = 0; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const float w = (float)(0.54 + 0.46 * cos(PI * (double)frac));
            F[i] = (revndim * (float)i) * w;
        }
        for (int i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_RAMP:
        for (int i = 0; i < ndimh; i++) F[i] = revndim * (float)i;
        for (int i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_PARZN:
        for (int i = 0; i < ndimh / 2; i++) {
            const float frac = (float)i / (float)ndimh;
            float t = 6.0f * frac;
            t = t * frac;
            t = t * (1.0f - frac);
            F[i] = (revndim * (float)i) * (1.0f - t);
        }
        for (int i = ndimh / 2; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const float om = 1.0f - frac;
            float v = (revndim * (float)i) * 2.0f;
            v = v * om;
            v = v * om;
            F[i] = v * om;
        }
        for (int i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    case RV_FILT_BUTER:
        for (int i = 0; i < ndim; i++) {
            const float frac = (float)i / (float)ndimh;
            const float den = sqrtf(1.0f + powf(frac, order));
            F[i] = (revndim * (float)i) / den;
        }
        break;
    case RV_FILT_SHEPP:
        for (int i = 0; i < ndimh; i++) {
            const float frac = (float)i / (float)ndimh;
            const double x = PI * (double)frac * 0.5;
            const float w = (i == 0) ? 1.0f : (float)(sin(x) / x);
            F[i] = (revndim * (float)i) * w;
        }
        for (int i = ndimh; i < ndim; i++) F[i] = 0;
        break;
    default:
        for (int i = 0; i < ndim; i++) F[i] = 1;
        break;
    }
    return 0;
}
