// Fused stack path (no reference counterpart): a whole dataset's raw uint16 frames for many
// detector rows -> normalised -> filtered -> back-projected slices, in a few launches.
//
// HBM layout (one stack, nslices slices of ixdimp^2, V back-projected views, W = ixdim):
//   raw      [(nframes+1) * nslices * W] uint16   the reference's sinogram buffer order
//   table    [batch * V * 16 * ixdimp]   int32    REF: 1/16 sub-sample tables, slice-major
//   rows     [batch * V * ixdimp]        f32/f16/bf16 LIN: filtered rows x100 (+ per-row scale)
//   out      [nslices * ixdimp^2]        int32 (REF) / f32 (LIN)
// Slices are processed in batches so the tables stay within a device-memory budget
// (RV_TABLE_BUDGET_MB, default 32768).
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "rv_internal.h"

using namespace rv;

struct RvStack {
    RvStackDesc desc{};
    Dims d{};
    int device = 0;
    int nviews = 0;                 // back-projected (SAMPLE) views
    int batch = 1;                  // slices per filter/back-projection batch
    std::vector<float> filt;
    std::vector<RowJob> jobs;       // slice-major: jobs[s * nviews + v]
    std::vector<float4> geom_ref;
    std::vector<LinGeom> geom_lin;
    void* d_jobs = nullptr;
    void* d_geom = nullptr;
    void* d_filt = nullptr;
    void* d_tw = nullptr;
    void* d_table = nullptr;        // REF tables or LIN rows
    void* d_scale = nullptr;
    void* d_in = nullptr;           // RunHost staging
    void* d_out = nullptr;
    size_t in_bytes = 0, out_bytes = 0;
    cudaEvent_t ev[6] = {};
    int nbatches_last = 0;
    float t_filter = 0, t_bp = 0, t_total = 0;
    int launches = 0;
    cudaStream_t cs_in = nullptr, cs_out = nullptr;   // RunHost copy streams
    cudaStream_t cs_alt = nullptr;                    // RunHost second compute stream
    std::vector<cudaEvent_t> pev;   // RunHost pipeline events
    int tfmt = 0;                   // REF table layout (ref_table_fmt at creation)
    float lin16_scale = 1.0f;       // FP16 rows: the power-of-two row scale of this filter
    long long tstride = 0;          // ints per table slot
};

static void stack_free(RvStack* st) {
    void* bufs[] = {st->d_jobs, st->d_geom, st->d_filt, st->d_tw, st->d_table, st->d_scale, st->d_in, st->d_out};
    for (void* p : bufs)
        if (p) cudaFree(p);
    for (cudaEvent_t& e : st->ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : st->pev)
        if (e) cudaEventDestroy(e);
    if (st->cs_in) cudaStreamDestroy(st->cs_in);
    if (st->cs_out) cudaStreamDestroy(st->cs_out);
    if (st->cs_alt) cudaStreamDestroy(st->cs_alt);
}

static int stack_create(const RvStackDesc* desc, RvStack** out, bool alloc_tables) {
    if (!desc || !out || !desc->bInc || !desc->fdeg || !desc->fFilter || desc->nframes < 1 || desc->nslices < 1 ||
        desc->ixdim < 4 || (!desc->input_is_sinogram && !desc->fexp) || desc->mode < RV_MODE_REF ||
        desc->mode > RV_MODE_LIN_BF16) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvStackCreate: invalid description");
        return RV_ERR_BAD_ARGUMENT;
    }
    if (desc->iRawWidth != 0) {
        // R2: source/gazoDoc.cpp:2987 (bin from iInterpolation), 3002-3004 (width)
        const int bin = desc->iInterpolation == 0 ? 4 : (desc->iInterpolation == 1 ? 2 : 1);
        const int F = desc->iRawWidth, T = desc->iTrim;
        const int want = (T >= 0 && (T == 0 || T < F / 2)) ? (F - (T > 0 ? 2 * T : 0)) / bin : -1;
        if (desc->input_is_sinogram || F < 0 || want < 0 || want != desc->ixdim) {
            set_error(RV_ERR_BAD_ARGUMENT, "RvStackCreate: iRawWidth/iTrim/binning do not give ixdim (width " +
                                               std::to_string(want) + ", ixdim " + std::to_string(desc->ixdim) +
                                               "), or the input is a sinogram");
            return RV_ERR_BAD_ARGUMENT;
        }
    } else if (desc->iTrim != 0) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvStackCreate: iTrim needs iRawWidth (the untrimmed frame width)");
        return RV_ERR_BAD_ARGUMENT;
    }
    RvStack* st = new RvStack();
    st->desc = *desc;
    st->d = make_dims(desc->ixdim, desc->iInterpolation);
    const Dims& d = st->d;
    if (d.ndimp > kMaxNdimp || d.ixdimp > kMaxIxdimp) {
        delete st;
        set_error(RV_ERR_UNSUPPORTED, "RvStackCreate: ixdim*zoom beyond 16384");
        return RV_ERR_UNSUPPORTED;
    }
    cudaGetDevice(&st->device);
    const int nf = desc->nframes, S = desc->nslices;
    const char* bInc = desc->bInc;
    // ---- views and their flats (GenerateSinogramThread bracketing, source/general.cpp:2415-2447)
    std::vector<int> views;
    std::vector<int> vi0, vi1;
    std::vector<float> vt0;
    std::vector<int> vzero;
    int i0 = -1, i1 = -1;
    for (int i = 0; i < nf; i++) {
        if (bInc[i] & RV_BINC_NOUSE) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; break; }
    }
    for (int i = 0; i < nf; i++) {
        if ((bInc[i] & RV_BINC_NOUSE) && !(bInc[i] & RV_BINC_SAMPLE)) continue;
        if (!(bInc[i] & RV_BINC_SAMPLE)) { i0 = i; i1 = -1; continue; }
        if (!desc->input_is_sinogram) {
            if (i1 < 0) {
                for (int j = i; j < nf; j++) {
                    if (bInc[j] & RV_BINC_SAMPLE) continue;
                    i1 = j;
                    break;
                }
                if (i1 < 0 && i0 >= 0) i1 = i0;
            }
            if (i0 < 0 || i1 < 0) {
                delete st;
                set_error(RV_ERR_BAD_ARGUMENT, "RvStackCreate: a sample frame has no flat frame");
                return RV_ERR_BAD_ARGUMENT;
            }
        }
        // back-projection selection (source/general.cpp:2087-2102)
        if (desc->dReconFlags & (RV_RQFLAGS_USEONLYEVENFRAMES | RV_RQFLAGS_USEONLYODDFRAMES)) {
            if (i & 1) {
                if (desc->dReconFlags & RV_RQFLAGS_USEONLYEVENFRAMES) continue;
            } else {
                if (desc->dReconFlags & RV_RQFLAGS_USEONLYODDFRAMES) continue;
            }
        }
        float t0 = 0.0f;
        if (!desc->input_is_sinogram) {
            t0 = desc->fexp[i0];
            const float t1 = desc->fexp[i1], ti = desc->fexp[i];
            if (t0 == t1) t0 = 0;
            else t0 = (ti - t0) / (t1 - t0);
        }
        views.push_back(i);
        vi0.push_back(i0);
        vi1.push_back(i1);
        vt0.push_back(t0);
        vzero.push_back((bInc[i] & RV_BINC_SKIP) ? 1 : 0);
    }
    st->nviews = (int)views.size();
    const int V = st->nviews;
    if (V == 0) {
        delete st;
        set_error(RV_ERR_BAD_ARGUMENT, "RvStackCreate: no sample frames");
        return RV_ERR_BAD_ARGUMENT;
    }
    // ---- geometry: REF in 1/16 units (reference order), LIN in detector pixels (from FP64) ----
    st->geom_ref.resize(V);
    st->geom_lin.resize(V);
    const double cen_lin = (double)d.ixdimh + (desc->center - (int)desc->center) * d.iIntpDim;
    for (int v = 0; v < V; v++) {
        float fc, fs, fo;
        view_geometry(d, desc->center, desc->fdeg[views[v]], desc->fTiltAngle, &fc, &fs, &fo);
        st->geom_ref[v] = make_float4(fc, fs, fo, ray_regime_tag(fc, fs));
        const double th = (double)(desc->fdeg[views[v]] + desc->fTiltAngle) * (3.14159265358979323846 / 180.0);
        const double c = cos(th), sn = -sin(th);
        st->geom_lin[v] = LinGeom{c, sn, cen_lin - d.ixdimh * (c + sn), 0.0};
    }
    st->filt.assign(desc->fFilter, desc->fFilter + d.ndim);
    st->lin16_scale = fp16_row_scale(st->filt.data(), d.ndim);
    // ---- batch size from the table budget ----------------------------------------------------
    size_t budget_mb = 32768;
    if (const char* e = getenv("RV_TABLE_BUDGET_MB")) budget_mb = (size_t)atoll(e);
    st->tfmt = ref_table_fmt();
    st->tstride = ref_table_stride(d.ixdimp, st->tfmt);
    const size_t per_slice = desc->mode == RV_MODE_REF
                                 ? (size_t)V * st->tstride * sizeof(int)
                                 : (size_t)V * lin_pair_stride(d.ixdimp) * lin_pair_bytes(desc->mode);
    size_t b = (budget_mb << 20) / (per_slice ? per_slice : 1);
    if (b < 1) b = 1;
    if (b > (size_t)S) b = S;
    st->batch = (int)b;
    // row jobs, slice-major; dst = slot inside the slice batch ((s mod batch) * V + v)
    st->jobs.resize((size_t)S * V);
    for (int s = 0; s < S; s++)
        for (int v = 0; v < V; v++) {
            RowJob j{};
            j.src_row = views[v] * S + s;
            j.flat0_row = vi0[v] * S + s;
            j.flat1_row = vi1[v] * S + s;
            j.dark_row = nf * S + s;
            j.t0 = vt0[v];
            j.zero = vzero[v];
            j.dst = (s % st->batch) * V + v;
            st->jobs[(size_t)s * V + v] = j;
        }
    // ---- device buffers -------------------------------------------------------------------------
    std::vector<float2> tw;
    fft_twiddles(d.ndimp, tw);
    bool ok = cuda_ok(cudaMalloc(&st->d_jobs, st->jobs.size() * sizeof(RowJob)), RV_ERR_DEVICE_OOM, "jobs") &&
              cuda_ok(cudaMalloc(&st->d_geom, (size_t)V * sizeof(LinGeom)), RV_ERR_DEVICE_OOM, "geometry") &&
              cuda_ok(cudaMalloc(&st->d_filt, (size_t)d.ndim * sizeof(float)), RV_ERR_DEVICE_OOM, "filter") &&
              cuda_ok(cudaMalloc(&st->d_tw, tw.size() * sizeof(float2)), RV_ERR_DEVICE_OOM, "twiddles") &&
              (!alloc_tables || cuda_ok(cudaMalloc(&st->d_table, per_slice * st->batch), RV_ERR_DEVICE_OOM, "tables")) &&
              cuda_ok(cudaMalloc(&st->d_scale, (size_t)st->batch * V * sizeof(float)), RV_ERR_DEVICE_OOM, "scales");
    if (ok) {
        const void* g = desc->mode == RV_MODE_REF ? (const void*)st->geom_ref.data() : (const void*)st->geom_lin.data();
        const size_t gbytes = (size_t)V * (desc->mode == RV_MODE_REF ? sizeof(float4) : sizeof(LinGeom));
        ok = cuda_ok(cudaMemcpy(st->d_jobs, st->jobs.data(), st->jobs.size() * sizeof(RowJob), cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "jobs") &&
             cuda_ok(cudaMemcpy(st->d_geom, g, gbytes, cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "geometry") &&
             cuda_ok(cudaMemcpy(st->d_filt, st->filt.data(), (size_t)d.ndim * sizeof(float), cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "filter") &&
             cuda_ok(cudaMemcpy(st->d_tw, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice), RV_ERR_COPY_H2D, "twiddles");
    }
    for (cudaEvent_t& e : st->ev)
        if (ok) ok = cuda_ok(cudaEventCreate(&e), RV_ERR_LAUNCH, "event");
    if (!ok) {
        const int code = RvGetLastError();
        stack_free(st);
        delete st;
        return code ? code : RV_ERR_DEVICE_OOM;
    }
    *out = st;
    return 0;
}

extern "C" int RvStackCreate(const RvStackDesc* desc, RvStack** out) { return stack_create(desc, out, true); }

extern "C" void RvStackDestroy(RvStack* st) {
    if (!st) return;
    cudaSetDevice(st->device);
    stack_free(st);
    delete st;
}

extern "C" size_t RvStackSliceBytes(const RvStack* st) {
    return st ? (size_t)st->d.ixdimp * st->d.ixdimp * 4 : 0;
}
// raw samples per logical row (one slice of one frame): ixdim, or bin detector rows of the
// untrimmed width when the library assembles the strips
static long long raw_row_samples(const RvStack* st) {
    if (st->desc.iRawWidth <= 0) return st->desc.ixdim;
    const int bin = st->desc.iInterpolation == 0 ? 4 : (st->desc.iInterpolation == 1 ? 2 : 1);
    return (long long)bin * st->desc.iRawWidth;
}
// the filter's view of the raw layout (R2 strip assembly)
static void set_raw_layout(const RvStack* st, FilterLaunch& fl) {
    if (st->desc.iRawWidth <= 0) return;
    fl.raw_stride = st->desc.iRawWidth;
    fl.raw_x0 = st->desc.iTrim;
    fl.bin = st->desc.iInterpolation == 0 ? 4 : (st->desc.iInterpolation == 1 ? 2 : 1);
}

extern "C" size_t RvStackInputBytes(const RvStack* st) {
    return st ? (size_t)(st->desc.nframes + 1) * st->desc.nslices * raw_row_samples(st) * 2 : 0;
}
extern "C" int RvStackNumViews(const RvStack* st) { return st ? st->nviews : 0; }
extern "C" int RvStackOutputDim(const RvStack* st) { return st ? st->d.ixdimp : 0; }

// Filter + back-projection of slices [s0, s0 + nb) (nb <= batch) on stream s; ev_a/ev_b/ev_c
// (may be null) bracket the two kernels.
static int run_slices(RvStack* st, const void* d_raw, void* d_out, int s0, int nb, cudaStream_t s, cudaEvent_t ev_a,
                      cudaEvent_t ev_b, cudaEvent_t ev_c) {
    const Dims& d = st->d;
    const int V = st->nviews, mode = st->desc.mode;
    const long long tstride = st->tstride;
    const size_t npix = (size_t)d.ixdimp * d.ixdimp;
    FilterLaunch fl{};
    fl.src = d_raw;
    fl.raw = st->desc.input_is_sinogram ? 0 : 1;
    set_raw_layout(st, fl);
    fl.pixmin = (st->desc.iFlag & RV_READTIF8bit) ? RV_SINOGRAM_PIXEL_MIN8bit : RV_SINOGRAM_PIXEL_MIN16bit;
    fl.jobs = static_cast<const RowJob*>(st->d_jobs) + (size_t)s0 * V;
    fl.njobs = nb * V;
    fl.filt = static_cast<const float*>(st->d_filt);
    fl.tw = static_cast<const float2*>(st->d_tw);
    fl.mode = mode;
    fl.d = d;
    fl.ic = (int)st->desc.center;
    if (mode == RV_MODE_REF) {
        fl.table = static_cast<int*>(st->d_table);
        fl.table_stride = tstride;
        fl.table_fmt = st->tfmt;
    } else {   // LIN forms: pair rows
        fl.rows16 = st->d_table;
        fl.row_scale = static_cast<float*>(st->d_scale);
        fl.row_stride = lin_pair_stride(d.ixdimp);
        fl.lin16_scale = st->lin16_scale;
    }
    // jobs of slice s write table slot (s mod batch): rebase so the first slice of this call
    // lands where its jobs point
    if (ev_a) cudaEventRecord(ev_a, s);
    cudaError_t e = launch_filter(fl, s);
    if (!cuda_ok(e, RV_ERR_LAUNCH, "filter kernel")) return RV_ERR_LAUNCH;
    if (ev_b) cudaEventRecord(ev_b, s);
    BackprojLaunch bl{};
    const size_t slot0 = (size_t)(s0 % st->batch);
    bl.table = static_cast<const int*>(st->d_table) + slot0 * (size_t)(tstride * V);
    const int lps = lin_pair_stride(d.ixdimp);
    bl.rows16 = static_cast<const char*>(st->d_table) + slot0 * (size_t)lps * V * lin_pair_bytes(mode);
    bl.row_scale = mode == RV_MODE_LIN_F16 || mode == RV_MODE_LIN_BF16 ? static_cast<const float*>(st->d_scale) + slot0 * V
                                                                       : nullptr;
    bl.geom = static_cast<const float4*>(st->d_geom);
    bl.geom64 = static_cast<const LinGeom*>(st->d_geom);
    bl.nviews = V;
    bl.nslices = nb;
    bl.ixdimp = d.ixdimp;
    bl.table_stride = tstride;
    bl.slice_table_stride = tstride * V;
    bl.row_stride = lps;
    bl.slice_row_stride = (long long)lps * V;
    bl.out = mode == RV_MODE_REF ? (void*)(static_cast<int*>(d_out) + (size_t)s0 * npix)
                                 : (void*)(static_cast<float*>(d_out) + (size_t)s0 * npix);
    bl.out_slice_stride = (long long)npix;
    bl.mode = mode;
    bl.table_fmt = st->tfmt;
    take_backproject_launches();
    e = launch_backproject(bl, s);
    if (!cuda_ok(e, RV_ERR_LAUNCH, "back-projection kernel")) return RV_ERR_LAUNCH;
    if (ev_c) cudaEventRecord(ev_c, s);
    st->launches += kernel_launches_per_filter() + take_backproject_launches();
    return 0;
}

extern "C" int RvStackRunDevice(RvStack* st, const void* d_raw, void* d_out, void* stream) {
    if (!st || !d_raw || !d_out) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvStackRunDevice: NULL argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int S = st->desc.nslices;
    st->launches = 0;
    float tf = 0, tb = 0;
    cudaEventRecord(st->ev[4], s);
    for (int s0 = 0; s0 < S; s0 += st->batch) {
        const int nb = (S - s0) < st->batch ? (S - s0) : st->batch;
        const int rc = run_slices(st, d_raw, d_out, s0, nb, s, st->ev[0], st->ev[1], st->ev[2]);
        if (rc) return rc;
        if (cudaEventSynchronize(st->ev[2]) == cudaSuccess) {
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, st->ev[0], st->ev[1]);
            cudaEventElapsedTime(&b, st->ev[1], st->ev[2]);
            tf += a;
            tb += b;
        }
    }
    cudaEventRecord(st->ev[5], s);
    cudaError_t e = cudaEventSynchronize(st->ev[5]);
    if (!cuda_ok(e, RV_ERR_LAUNCH, "stack run")) return RV_ERR_LAUNCH;
    if (const unsigned ks = take_kernel_status(s)) {
        set_error(RV_ERR_KERNEL_STATUS, std::string("back-projection: ") + kernel_status_text(ks));
        return RV_ERR_KERNEL_STATUS;
    }
    float tt = 0;
    cudaEventElapsedTime(&tt, st->ev[4], st->ev[5]);
    st->t_filter = tf;
    st->t_bp = tb;
    st->t_total = tt;
    return 0;
}

// Host-buffer run, pipelined: the slices are processed in pieces; piece k's frames (all frames,
// the piece's detector rows: one strided 2-D copy) go up on an input copy stream, its filter and
// back-projection run on the caller's stream or (odd pieces) a second compute stream, and its
// slices come back on an output copy stream, so host<->device traffic and the tail of one
// piece's back-projection overlap the work of neighbouring pieces.
static int ensure_host_buffers(RvStack* st, size_t in_b, size_t out_b) {
    if (st->in_bytes < in_b) {
        if (st->d_in) cudaFree(st->d_in);
        st->d_in = nullptr;
        st->in_bytes = 0;
        if (!cuda_ok(cudaMalloc(&st->d_in, in_b), RV_ERR_DEVICE_OOM, "input buffer")) return RV_ERR_DEVICE_OOM;
        st->in_bytes = in_b;
    }
    if (st->out_bytes < out_b) {
        if (st->d_out) cudaFree(st->d_out);
        st->d_out = nullptr;
        st->out_bytes = 0;
        if (!cuda_ok(cudaMalloc(&st->d_out, out_b), RV_ERR_DEVICE_OOM, "output buffer")) return RV_ERR_DEVICE_OOM;
        st->out_bytes = out_b;
    }
    if (!st->cs_in) {
        if (!cuda_ok(cudaStreamCreateWithFlags(&st->cs_in, cudaStreamNonBlocking), RV_ERR_STREAM, "copy stream") ||
            !cuda_ok(cudaStreamCreateWithFlags(&st->cs_out, cudaStreamNonBlocking), RV_ERR_STREAM, "copy stream") ||
            !cuda_ok(cudaStreamCreateWithFlags(&st->cs_alt, cudaStreamNonBlocking), RV_ERR_STREAM, "compute stream"))
            return RV_ERR_STREAM;
    }
    return 0;
}

// Slices per piece of the host pipeline: about S / 16 (RV_STACK_PIECES pieces), rounded up to
// whole slice groups of the default back-projection (three slices per CTA for variant 21, else
// two), at most one table batch.  Pieces never straddle two table batches (slots s mod batch):
// each batch is cut into pieces of this size, its last piece possibly shorter.
static int piece_slices(const RvStack* st) {
    int pieces = 16;
    if (const char* e = getenv("RV_STACK_PIECES")) pieces = atoi(e);
    const int S = st->desc.nslices;
    if (pieces < 1) pieces = 1;
    int p = (S + pieces - 1) / pieces;
    const int g = default_variant() == 21 ? 3 : 2;
    p = (p + g - 1) / g * g;
    if (p > st->batch) p = st->batch;
    if (p < 1) p = 1;
    return p;
}
// piece k: slices [*s0, *s0 + *nb) (nb = 0 past the end); ppw pieces per table batch
static void piece_range(const RvStack* st, int P, int ppw, int k, int* s0, int* nb) {
    const int S = st->desc.nslices;
    const int w = k / ppw, j = k % ppw;
    *s0 = w * st->batch + j * P;
    int n = P;
    if (j * P + n > st->batch) n = st->batch - j * P;
    if (*s0 + n > S) n = S - *s0;
    *nb = n > 0 ? n : 0;
}

extern "C" int RvStackRunHost(RvStack* st, const void* h_raw, void* h_out, void* stream) {
    if (!st || !h_raw || !h_out) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvStackRunHost: NULL argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int S = st->desc.nslices, nfr = st->desc.nframes + 1;
    const size_t W = (size_t)raw_row_samples(st);   // raw samples per slice of a frame
    const size_t in_b = RvStackInputBytes(st);
    const size_t slice_b = RvStackSliceBytes(st);
    int rc = ensure_host_buffers(st, in_b, slice_b * S);
    if (rc) return rc;
    const int P = piece_slices(st);
    const int ppw = (st->batch + P - 1) / P;   // pieces per table batch; piece k reuses piece k - ppw's slots
    int npieces = 0;
    for (int s0 = 0, nb = 1; nb > 0; npieces++) {
        piece_range(st, P, ppw, npieces, &s0, &nb);
        if (nb == 0) break;
    }
    // events: start, per piece {in copied, filter start, filter end, bp end, out copied}, end
    const size_t need = 2 + 5 * (size_t)npieces;
    while (st->pev.size() < need) {
        cudaEvent_t e = nullptr;
        if (!cuda_ok(cudaEventCreate(&e), RV_ERR_LAUNCH, "event")) return RV_ERR_LAUNCH;
        st->pev.push_back(e);
    }
    cudaEvent_t* E = st->pev.data();
    st->launches = 0;
    // the copy streams start after earlier work of the caller's stream on these buffers
    cudaEventRecord(E[0], s);
    cudaStreamWaitEvent(st->cs_in, E[0], 0);
    cudaStreamWaitEvent(st->cs_out, E[0], 0);
    cudaStreamWaitEvent(st->cs_alt, E[0], 0);
    const size_t pitch = (size_t)S * W * 2;
    const int reuse = ppw;   // pieces later a piece's table slots come round again
    for (int k = 0; k < npieces; k++) {
        int s0 = 0, nb = 0;
        piece_range(st, P, ppw, k, &s0, &nb);
        cudaEvent_t* e = E + 1 + 5 * (size_t)k;
        const char* src = static_cast<const char*>(h_raw) + (size_t)s0 * W * 2;
        char* dst = static_cast<char*>(st->d_in) + (size_t)s0 * W * 2;
        if (!cuda_ok(cudaMemcpy2DAsync(dst, pitch, src, pitch, (size_t)nb * W * 2, nfr, cudaMemcpyHostToDevice,
                                       st->cs_in), RV_ERR_COPY_H2D, "raw frames"))
            return RV_ERR_COPY_H2D;
        cudaEventRecord(e[0], st->cs_in);
        // consecutive pieces alternate between two compute streams, so one piece's filter (and the
        // start of its back-projection) fills the SMs the previous back-projection's last wave leaves
        cudaStream_t ks = (k & 1) ? st->cs_alt : s;
        cudaStreamWaitEvent(ks, e[0], 0);
        if (k >= reuse) cudaStreamWaitEvent(ks, E[1 + 5 * (size_t)(k - reuse) + 3], 0);   // its table slots are free
        rc = run_slices(st, st->d_in, st->d_out, s0, nb, ks, e[1], e[2], e[3]);
        if (rc) return rc;
        cudaStreamWaitEvent(st->cs_out, e[3], 0);
        if (!cuda_ok(cudaMemcpyAsync(static_cast<char*>(h_out) + (size_t)s0 * slice_b,
                                     static_cast<const char*>(st->d_out) + (size_t)s0 * slice_b, (size_t)nb * slice_b,
                                     cudaMemcpyDeviceToHost, st->cs_out), RV_ERR_COPY_D2H, "slices"))
            return RV_ERR_COPY_D2H;
        cudaEventRecord(e[4], st->cs_out);
    }
    // the caller's stream (and so a later call) waits for the last copy back
    cudaEvent_t end = E[1 + 5 * (size_t)npieces];
    cudaStreamWaitEvent(s, E[5 * (size_t)npieces], 0);
    cudaEventRecord(end, s);
    if (!cuda_ok(cudaEventSynchronize(end), RV_ERR_COPY_D2H, "stack run")) return RV_ERR_COPY_D2H;
    if (const unsigned ks = take_kernel_status(s)) {
        set_error(RV_ERR_KERNEL_STATUS, std::string("back-projection: ") + kernel_status_text(ks));
        return RV_ERR_KERNEL_STATUS;
    }
    float tf = 0, tb = 0, tt = 0;
    for (int k = 0; k < npieces; k++) {
        cudaEvent_t* e = E + 1 + 5 * (size_t)k;
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, e[1], e[2]);
        cudaEventElapsedTime(&b, e[2], e[3]);
        tf += a;
        tb += b;
    }
    cudaEventElapsedTime(&tt, E[0], end);
    st->t_filter = tf;
    st->t_bp = tb;
    st->t_total = tt;
    return 0;
}

extern "C" int RvStackLastTimings(const RvStack* st, float* ms3) {
    if (!st || !ms3) return RV_ERR_BAD_ARGUMENT;
    ms3[0] = st->t_filter;
    ms3[1] = st->t_bp;
    ms3[2] = st->t_total;
    return 0;
}

extern "C" int RvStackLastLaunchCount(const RvStack* st) { return st ? st->launches : 0; }

// =============================================================================================
// Batched queue (no reference counterpart; replaces the sequential item loop of
// source/DlgQueue.cpp:363-470 and CGazoDoc::BatchReconst, source/gazoDoc.cpp:1938-1993).
// Datasets of uneven width, view count, centre and zoom are added as stacks; RvQueueRun groups
// (dataset, slice) pairs into waves whose int tables fit a device-memory pool, and each wave is
// one filter launch per dataset plus ONE persistent back-projection launch that takes 64x64 (or
// the tuned shape) tiles from a device work list until it is empty.  The whole sequence is
// captured once into a CUDA graph and replayed on later runs.
// =============================================================================================
struct RvQueueItem {
    RvStack* st;
    const void* d_raw;
    void* d_out;
    int variant;   // back-projection variant of this dataset's tiles (-1: the queue's default)
};

// ---- per-shape autotuning --------------------------------------------------------------------
// A dataset's shape class: output size (ixdimp <= 1024 / 2048 / 4096 / more), view count
// (<= 1000 / 2000 / more), whether its slices can run as pairs (two or more slices), and the
// table layout.  RvQueueAutotune times candidate persistent variants -- they differ in pixel tile
// (64x64, 128x64, 128x128), views per staged chunk, slices per CTA (1 or 2) and consumer warps
// (8 or 16) -- on a few slices of one dataset of each class, and the winner is kept in a
// process-wide cache keyed by the class, so later queues with the same shapes reuse it.
static unsigned shape_key(const RvStack* st, int fmt) {
    const int n = st->d.ixdimp, V = st->nviews;
    const unsigned cx = n <= 1024 ? 0u : (n <= 2048 ? 1u : (n <= 4096 ? 2u : 3u));
    const unsigned cv = V <= 1000 ? 0u : (V <= 2000 ? 1u : 2u);
    const unsigned pr = st->desc.nslices >= 2 ? 1u : 0u;
    return cx | (cv << 2) | (pr << 4) | ((unsigned)fmt << 5);
}
static std::mutex g_shape_mu;
static std::map<unsigned, int> g_shape_variant;
static int cached_variant(unsigned key) {
    std::lock_guard<std::mutex> lock(g_shape_mu);
    auto it = g_shape_variant.find(key);
    return it == g_shape_variant.end() ? -1 : it->second;
}

struct RvQueue {
    std::vector<RvQueueItem> items;
    int fmt = kTabInt16;
    int variant = -1;   // default variant for datasets whose shape class has no tuned choice
    bool built = false;
    // one back-projection per variant group of a wave: a persistent launch over the group's tile
    // list, or -- for groups with many tiles, where a work list gains nothing over the hardware's
    // own scheduling -- the regular grid launch of each part (grid non-empty)
    struct Group { int variant = 0, tile_begin = 0, ntiles = 0; std::vector<BackprojLaunch> grid; };
    struct Wave { std::vector<FilterLaunch> filters; std::vector<Group> groups; };
    std::vector<Wave> waves;
    void* d_rowjobs = nullptr;
    void* d_tiles = nullptr;
    void* d_pool = nullptr;
    unsigned* d_counters = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev[2] = {};
    float last_ms = 0;
    size_t total_tiles = 0;
    double total_updates = 0;
    void release_plan() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        void* b[] = {d_rowjobs, d_tiles, d_pool, d_counters};
        for (void* p : b)
            if (p) cudaFree(p);
        d_rowjobs = d_tiles = d_pool = nullptr;
        d_counters = nullptr;
        waves.clear();
        built = false;
    }
    int item_variant(int it) const { return items[it].variant >= 0 ? items[it].variant : variant; }
};

extern "C" int RvQueueCreate(RvQueue** out) {
    if (!out) return RV_ERR_BAD_ARGUMENT;
    RvQueue* q = new RvQueue();
    const int f = ref_table_fmt();
    q->fmt = (f == kTabInt17) ? kTabInt17 : kTabInt16;
    q->variant = default_variant();
    if (!cuda_ok(cudaEventCreate(&q->ev[0]), RV_ERR_LAUNCH, "event") ||
        !cuda_ok(cudaEventCreate(&q->ev[1]), RV_ERR_LAUNCH, "event")) {
        delete q;
        return RV_ERR_LAUNCH;
    }
    *out = q;
    return 0;
}

extern "C" int RvQueueAdd(RvQueue* q, const RvStackDesc* desc, const void* d_raw, void* d_out) {
    if (!q || !desc || !d_raw || !d_out) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvQueueAdd: NULL argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    if (desc->mode != RV_MODE_REF) {
        set_error(RV_ERR_UNSUPPORTED, "RvQueueAdd: the queue runs the reference-semantics mode only");
        return RV_ERR_UNSUPPORTED;
    }
    RvStack* st = nullptr;   // the queue keeps its own table pool: no per-stack tables
    const int rc = stack_create(desc, &st, false);
    if (rc) return rc;
    q->items.push_back({st, d_raw, d_out, cached_variant(shape_key(st, q->fmt))});
    q->release_plan();
    return 0;
}

// slices [s0, s1) of item `item`, back-projected with `variant`
struct QueueReq { int item, s0, s1, variant; };
// tiles of a variant group from which the wave launches the regular grid kernels instead of the
// persistent one (about eight waves of 64x64 tiles on the GPU; RV_QUEUE_GRID_TILES overrides)
static int grid_tiles_threshold() {
    const char* e = getenv("RV_QUEUE_GRID_TILES");
    return e ? atoi(e) : 2432;
}

static int queue_build_reqs(RvQueue* q, const std::vector<QueueReq>& reqs) {
    q->release_plan();
    q->total_updates = 0;
    size_t budget_mb = 32768;
    if (const char* e = getenv("RV_TABLE_BUDGET_MB")) budget_mb = (size_t)atoll(e);
    const size_t pool_words_max = (budget_mb << 20) / 4;
    // ---- waves of (item, slice range) whose tables fit the pool ---------------------------
    struct Part { int item, s0, s1, variant; size_t off; };
    std::vector<std::vector<Part>> wparts(1);
    size_t used = 0, pool_words = 0;
    for (const QueueReq& rq : reqs) {
        RvStack* st = q->items[rq.item].st;
        const size_t per_slice = (size_t)st->nviews * (size_t)ref_table_stride(st->d.ixdimp, q->fmt);
        if (per_slice > pool_words_max) {
            set_error(RV_ERR_UNSUPPORTED, "RvQueueRun: one slice's tables exceed the table budget");
            return RV_ERR_UNSUPPORTED;
        }
        int s = rq.s0;
        while (s < rq.s1) {
            if (used + per_slice > pool_words_max) {
                wparts.emplace_back();
                used = 0;
            }
            int n = (int)((pool_words_max - used) / per_slice);
            if (n > rq.s1 - s) n = rq.s1 - s;
            wparts.back().push_back({rq.item, s, s + n, rq.variant, used});
            used += per_slice * n;
            if (used > pool_words) pool_words = used;
            s += n;
        }
    }
    // ---- row jobs, filter launches and tile work lists (tiles grouped by variant) ------------
    std::vector<RowJob> rowjobs;
    std::vector<TileJob> tiles;
    std::vector<size_t> rj_begin;   // per filter launch: start index into rowjobs
    for (auto& parts : wparts) {
        RvQueue::Wave w;
        for (const Part& pt : parts) {
            RvStack* st = q->items[pt.item].st;
            const int V = st->nviews;
            const long long ts = ref_table_stride(st->d.ixdimp, q->fmt);
            rj_begin.push_back(rowjobs.size());
            for (int sl = pt.s0; sl < pt.s1; sl++)
                for (int v = 0; v < V; v++) {
                    RowJob j = st->jobs[(size_t)sl * V + v];
                    j.dst = (sl - pt.s0) * V + v;
                    rowjobs.push_back(j);
                }
            FilterLaunch fl{};
            fl.src = q->items[pt.item].d_raw;
            fl.raw = st->desc.input_is_sinogram ? 0 : 1;
            set_raw_layout(st, fl);
            fl.pixmin = (st->desc.iFlag & RV_READTIF8bit) ? RV_SINOGRAM_PIXEL_MIN8bit : RV_SINOGRAM_PIXEL_MIN16bit;
            fl.njobs = (pt.s1 - pt.s0) * V;
            fl.filt = static_cast<const float*>(st->d_filt);
            fl.tw = static_cast<const float2*>(st->d_tw);
            fl.table = reinterpret_cast<int*>((size_t)pt.off * 4);   // pool offset, rebased below
            fl.mode = RV_MODE_REF;
            fl.d = st->d;
            fl.ic = (int)st->desc.center;
            fl.table_stride = ts;
            fl.table_fmt = q->fmt;
            w.filters.push_back(fl);
        }
        // tiles: every part of a variant forms one group (one persistent launch)
        std::vector<int> variants;
        for (const Part& pt : parts)
            if (std::find(variants.begin(), variants.end(), pt.variant) == variants.end()) variants.push_back(pt.variant);
        for (int var : variants) {
            RvQueue::Group g;
            g.variant = var;
            g.tile_begin = (int)tiles.size();
            int tx = 64, ty = 64;
            persistent_tile_xy(var, &tx, &ty);
            // the slice-group kernels take two (18-20) or three (21, the rest of a part as pairs)
            // consecutive slices of a part per job: they share the geometry and their tables
            // follow each other in the pool
            const int group = (var >= 18 && var <= 20) ? 2 : (var == 21 ? 3 : 1);
            for (const Part& pt : parts) {
                if (pt.variant != var) continue;
                RvStack* st = q->items[pt.item].st;
                const int V = st->nviews;
                const long long ts = ref_table_stride(st->d.ixdimp, q->fmt);
                const size_t npix = (size_t)st->d.ixdimp * st->d.ixdimp;
                const int ntx = (st->d.ixdimp + tx - 1) / tx, nty = (st->d.ixdimp + ty - 1) / ty;
                // slices per job: groups of `group`, a triple part's rest as pairs (n = 3t,
                // 3t + 2, 3(t - 1) + 4), a single slice only when the part has one
                const int n = pt.s1 - pt.s0;
                int t3 = group == 3 ? n / 3 : 0;
                if (group == 3 && n % 3 == 1 && t3 > 0) t3--;
                for (int sl = pt.s0, step = 1; sl < pt.s1; sl += step) {
                    const int done = sl - pt.s0;
                    step = group == 3 ? (done < 3 * t3 ? 3 : 2) : group;
                    if (step > pt.s1 - sl) step = pt.s1 - sl;
                    for (int t = 0; t < ntx * nty; t++) {
                        TileJob J{};
                        J.table = reinterpret_cast<const int*>((pt.off + (size_t)(sl - pt.s0) * V * ts) * 4);
                        J.geom = static_cast<const float4*>(st->d_geom);
                        J.out = static_cast<int*>(q->items[pt.item].d_out) + (size_t)sl * npix;
                        J.table_stride = ts;
                        J.nviews = V;
                        J.ixdimp = st->d.ixdimp;
                        J.X0 = (t % ntx) * tx;
                        J.Y0 = (t / ntx) * ty;
                        J.pair = step - 1;
                        tiles.push_back(J);
                    }
                }
                q->total_updates += (double)(pt.s1 - pt.s0) * V * npix;
            }
            g.ntiles = (int)tiles.size() - g.tile_begin;
            if (g.ntiles >= grid_tiles_threshold()) {
                // large group: regular launches per part (tables at the part's pool offset)
                for (const Part& pt : parts) {
                    if (pt.variant != var) continue;
                    RvStack* st = q->items[pt.item].st;
                    const long long ts = ref_table_stride(st->d.ixdimp, q->fmt);
                    const size_t npix = (size_t)st->d.ixdimp * st->d.ixdimp;
                    BackprojLaunch bl{};
                    bl.table = reinterpret_cast<const int*>((size_t)pt.off * 4);   // rebased below
                    bl.geom = static_cast<const float4*>(st->d_geom);
                    bl.nviews = st->nviews;
                    bl.nslices = pt.s1 - pt.s0;
                    bl.ixdimp = st->d.ixdimp;
                    bl.table_stride = ts;
                    bl.slice_table_stride = ts * st->nviews;
                    bl.out = static_cast<int*>(q->items[pt.item].d_out) + (size_t)pt.s0 * npix;
                    bl.out_slice_stride = (long long)npix;
                    bl.mode = RV_MODE_REF;
                    bl.table_fmt = q->fmt;
                    g.grid.push_back(bl);
                }
            }
            w.groups.push_back(g);
        }
        q->waves.push_back(std::move(w));
    }
    size_t ngroups = 0;
    for (const auto& w : q->waves) ngroups += w.groups.size();
    q->total_tiles = tiles.size();
    if (!cuda_ok(cudaMalloc(&q->d_pool, pool_words * 4 + 16), RV_ERR_DEVICE_OOM, "table pool") ||
        !cuda_ok(cudaMalloc(&q->d_rowjobs, rowjobs.size() * sizeof(RowJob) + 16), RV_ERR_DEVICE_OOM, "row jobs") ||
        !cuda_ok(cudaMalloc(&q->d_tiles, tiles.size() * sizeof(TileJob) + 16), RV_ERR_DEVICE_OOM, "tiles") ||
        !cuda_ok(cudaMalloc((void**)&q->d_counters, (ngroups + 1) * sizeof(unsigned)), RV_ERR_DEVICE_OOM, "counters"))
        return RvGetLastError();
    // rebase pool offsets to device addresses
    int* pool = static_cast<int*>(q->d_pool);
    for (TileJob& J : tiles) J.table = pool + reinterpret_cast<size_t>(J.table) / 4;
    for (auto& w : q->waves)
        for (RvQueue::Group& g : w.groups)
            for (BackprojLaunch& bl : g.grid) bl.table = pool + reinterpret_cast<size_t>(bl.table) / 4;
    size_t fi = 0;
    for (auto& w : q->waves)
        for (FilterLaunch& fl : w.filters) {
            fl.table = pool + reinterpret_cast<size_t>(fl.table) / 4;
            fl.jobs = static_cast<const RowJob*>(q->d_rowjobs) + rj_begin[fi++];
        }
    if (!cuda_ok(cudaMemcpy(q->d_rowjobs, rowjobs.data(), rowjobs.size() * sizeof(RowJob), cudaMemcpyHostToDevice),
                 RV_ERR_COPY_H2D, "row jobs") ||
        !cuda_ok(cudaMemcpy(q->d_tiles, tiles.data(), tiles.size() * sizeof(TileJob), cudaMemcpyHostToDevice),
                 RV_ERR_COPY_H2D, "tiles"))
        return RvGetLastError();
    q->built = true;
    return 0;
}

// the whole queue: every dataset's slices with its own variant
static int queue_build(RvQueue* q) {
    std::vector<QueueReq> reqs;
    for (int it = 0; it < (int)q->items.size(); it++)
        reqs.push_back({it, 0, q->items[it].st->desc.nslices, q->item_variant(it)});
    return queue_build_reqs(q, reqs);
}

static int queue_launch(RvQueue* q, cudaStream_t s) {
    const TileJob* tiles = static_cast<const TileJob*>(q->d_tiles);
    size_t c = 0;
    for (size_t w = 0; w < q->waves.size(); w++) {
        RvQueue::Wave& wv = q->waves[w];
        if (!wv.groups.empty() &&
            !cuda_ok(cudaMemsetAsync(q->d_counters + c, 0, wv.groups.size() * sizeof(unsigned), s), RV_ERR_MEMSET,
                     "counter"))
            return RV_ERR_MEMSET;
        for (const FilterLaunch& fl : wv.filters)
            if (!cuda_ok(launch_filter(fl, s), RV_ERR_LAUNCH, "filter kernel")) return RV_ERR_LAUNCH;
        for (const RvQueue::Group& g : wv.groups) {
            if (!g.grid.empty()) {
                for (const BackprojLaunch& bl : g.grid)
                    if (!cuda_ok(launch_bp_ref_variant(bl, s, g.variant), RV_ERR_LAUNCH, "back-projection"))
                        return RV_ERR_LAUNCH;
            } else if (!cuda_ok(launch_bp_ref_persistent(tiles + g.tile_begin, g.ntiles, q->d_counters + c, q->fmt,
                                                         g.variant, s),
                                RV_ERR_LAUNCH, "persistent back-projection")) {
                return RV_ERR_LAUNCH;
            }
            c++;
        }
    }
    return 0;
}

extern "C" int RvQueueRun(RvQueue* q, void* stream) {
    if (!q) return RV_ERR_BAD_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    cudaStream_t cap = nullptr;
    int rc = 0;
    if (!q->built) {
        if ((rc = queue_build(q))) return rc;
        // capture the whole sequence once (on a private stream: the legacy stream cannot capture)
        if (!cuda_ok(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), RV_ERR_STREAM, "capture stream"))
            return RV_ERR_STREAM;
        if (!cuda_ok(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), RV_ERR_LAUNCH, "graph capture")) {
            cudaStreamDestroy(cap);
            return RV_ERR_LAUNCH;
        }
        rc = queue_launch(q, cap);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (!cuda_ok(e, RV_ERR_LAUNCH, "graph capture") ||
            !cuda_ok(cudaGraphInstantiate(&q->exec, g, 0), RV_ERR_LAUNCH, "graph instantiate")) {
            if (g) cudaGraphDestroy(g);
            return RV_ERR_LAUNCH;
        }
        q->graph = g;
    }
    cudaEventRecord(q->ev[0], s);
    if (!cuda_ok(cudaGraphLaunch(q->exec, s), RV_ERR_LAUNCH, "graph launch")) return RV_ERR_LAUNCH;
    cudaEventRecord(q->ev[1], s);
    if (!cuda_ok(cudaEventSynchronize(q->ev[1]), RV_ERR_LAUNCH, "queue run")) return RV_ERR_LAUNCH;
    cudaEventElapsedTime(&q->last_ms, q->ev[0], q->ev[1]);
    if (const unsigned ks = take_kernel_status(s)) {
        set_error(RV_ERR_KERNEL_STATUS, std::string("back-projection: ") + kernel_status_text(ks));
        return RV_ERR_KERNEL_STATUS;
    }
    return 0;
}

// device time of one plan launch (after one untimed launch), in ms; < 0 on error
static float time_plan(RvQueue* q, cudaStream_t s, int reps) {
    if (queue_launch(q, s)) return -1.0f;
    float best = 3.0e38f;
    for (int r = 0; r < reps; r++) {
        cudaEventRecord(q->ev[0], s);
        if (queue_launch(q, s)) return -1.0f;
        cudaEventRecord(q->ev[1], s);
        if (cudaEventSynchronize(q->ev[1]) != cudaSuccess) return -1.0f;
        float ms = 0;
        cudaEventElapsedTime(&ms, q->ev[0], q->ev[1]);
        if (ms < best) best = ms;
    }
    return best;
}

extern "C" int RvQueueAutotune(RvQueue* q, void* stream, int* chosen) {
    // per shape class of the queue's datasets: time each candidate variant's persistent kernel on
    // a few slices of the first dataset of the class, keep the fastest in the process-wide cache
    // and in every dataset of the class
    if (!q || q->items.empty()) return RV_ERR_BAD_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    // candidates spanning the tuned dimensions: 64x64 tiles with three-slice groups and 3-view
    // chunks (21; the rest of a dataset as pairs), slice pairs with 16 consumer warps (19), single
    // slices with 6-view chunks (16), compact
    // lane blocks (17), warp-0-produced pipelines with 4- and 5-view chunks (11, 14), 128x128 and
    // 128x64 tiles (0, 4)
    const int cands[] = {21, 19, 16, 17, 11, 14, 0, 4};
    std::map<unsigned, int> tuned;
    for (int it = 0; it < (int)q->items.size(); it++) {
        const unsigned key = shape_key(q->items[it].st, q->fmt);
        if (tuned.count(key)) continue;
        // probe slices: enough 64x64 tiles to fill the GPU about twice (2..8 slices, even when
        // the class runs slice pairs), never more than the dataset has
        const int S = q->items[it].st->desc.nslices;
        const int t64 = ((q->items[it].st->d.ixdimp + 63) / 64) * ((q->items[it].st->d.ixdimp + 63) / 64);
        int n = (2048 + t64 - 1) / t64;
        n = n < 2 ? 2 : (n > 8 ? 8 : n);
        n += n & 1;
        if (n > S) n = S;
        float best = 3.0e38f;
        int bestv = q->variant;
        for (int v : cands) {
            const int rc = queue_build_reqs(q, {QueueReq{it, 0, n, v}});
            if (rc) return rc;
            const float ms = time_plan(q, s, 2);
            if (ms < 0.0f) {
                q->release_plan();
                set_error(RV_ERR_LAUNCH, "RvQueueAutotune: a probe launch failed");
                return RV_ERR_LAUNCH;
            }
            if (ms < best) {
                best = ms;
                bestv = v;
            }
        }
        tuned[key] = bestv;
        std::lock_guard<std::mutex> lock(g_shape_mu);
        g_shape_variant[key] = bestv;
    }
    for (RvQueueItem& item : q->items) item.variant = tuned[shape_key(item.st, q->fmt)];
    q->release_plan();
    if (const unsigned ks = take_kernel_status(s)) {
        set_error(RV_ERR_KERNEL_STATUS, std::string("back-projection: ") + kernel_status_text(ks));
        return RV_ERR_KERNEL_STATUS;
    }
    if (chosen) *chosen = q->items[0].variant;
    return 0;
}

extern "C" int RvQueueSetItemVariant(RvQueue* q, int item, int variant) {
    // every int-table variant 0..21 has a persistent form
    if (!q || item < 0 || item >= (int)q->items.size() || variant < 0 || variant > 21) return RV_ERR_BAD_ARGUMENT;
    q->items[item].variant = variant;
    q->release_plan();
    return 0;
}

extern "C" int RvQueueItemVariant(const RvQueue* q, int item) {
    if (!q || item < 0 || item >= (int)q->items.size()) return -1;
    return q->item_variant(item);
}

extern "C" float RvQueueLastMs(const RvQueue* q) { return q ? q->last_ms : 0.0f; }
extern "C" double RvQueueUpdates(const RvQueue* q) { return q ? q->total_updates : 0.0; }

extern "C" void RvQueueDestroy(RvQueue* q) {
    if (!q) return;
    q->release_plan();
    for (RvQueueItem& it : q->items) RvStackDestroy(it.st);
    for (cudaEvent_t& e : q->ev)
        if (e) cudaEventDestroy(e);
    delete q;
}
