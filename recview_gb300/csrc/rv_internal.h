// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/recview_gb300.h"

namespace rv {

// ---- error reporting ---------------------------------------------------------------------
void set_error(int code, const std::string& msg);
inline bool cuda_ok(cudaError_t e, int code, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

// ---- per-context state ----------------------------------------------------------------------
// Identifier of the CUDA context current on the calling thread: unique for the life of the
// process, so a device reset (which destroys the context and every device address resolved in
// it) always yields a new value.  0 when no live context is current or the driver cannot say.
// Host-side caches of device addresses or one-time device fills are keyed by it.
unsigned long long current_context_id();

// ---- geometry ----------------------------------------------------------------------------
struct Dims {
    int ixdim, iZooming, iIntpDim, ndimp, ndim, ixdimp, ixdimh, ihoffset;
};
Dims make_dims(int ixdim, int iInterpolation);
// float geometry of one view in the reference's operation order (source/general.cpp:2139-2142)
float fcenter_of(const Dims& d, double center);
void view_geometry(const Dims& d, double center, float fdeg, float tilt, float* fcos, float* fsin,
                   float* foffset);
// twiddles of CFft::Init1(np, -1), correctly rounded, laid out per radix-2 pass: entry 2^l + q
// holds w[q << (np-1-l)] (n entries; 0 and 1 unused)
void fft_twiddles(int np, std::vector<float2>& out);

// limits of the on-chip FFT and of the back-projection tile windows
constexpr int kMaxNdimp = 14;        // ndim <= 16384 (one row per CTA in shared memory)
constexpr int kMaxIxdimp = 16384;    // 16 * ixdimp < 2^23 keeps the exact truncation trick valid

// ---- per-row job of the filter stage -------------------------------------------------------
// One filtered row = one (view, slice).  Source rows are either int16 sinogram rows or raw
// uint16 frames normalised on the fly against flats i0/i1 (weight t0) and the dark row.
struct RowJob {
    int src_row;     // row index of the sample (int16 sinogram or raw uint16 frame row)
    int flat0_row;   // raw mode: bracketing flat rows and dark row
    int flat1_row;
    int dark_row;
    float t0;        // raw mode: flat interpolation weight (source/general.cpp:2443-2447)
    int dst;         // output slot (view-major within a slice: slice * nviews + v)
    int zero;        // 1: the row is all zero (SKIP frame)
    int ic;          // integer centre of this row when FilterLaunch::ic_per_job is set
};

struct FilterLaunch {
    const void* src;          // int16 rows or uint16 raw rows, row stride = ixdim elements
    int raw;                  // 1: src holds raw uint16 frames (normalise), 0: int16 sinogram
    int pixmin;               // sample threshold (source/general.cpp:2402)
    const RowJob* jobs;       // device array
    int njobs;
    const float* filt;        // device, ndim
    const float2* tw;         // device, ndim entries: pass l's twiddle q at [2^l + q]
    int* table;               // REF output: int table, 16*ixdimp ints per slot (may be null)
    void* rows16;             // LIN output: pair rows (r, r[j+1]-r) x BACKPROJ_SCALE, FP32 / FP16 / BF16
    float* row_scale;         // per-row scale of the 16-bit pair rows
    int mode;
    Dims d;
    int ic;                   // (int)center
    int ic_per_job;           // 1: take the integer centre from each RowJob (centre sweeps)
    long long table_stride;   // ints between table slots
    long long row_stride;     // pairs between LIN rows (lin_pair_stride)
    int table_fmt;            // REF table format, see ref_table_fmt()
    const short* const* row_ptr;  // sinogram mode: if set, row j is row_ptr[job.src_row] (it may be
                                  // host memory the device reads directly) instead of src + j * ixdim
    // raw mode, strip assembly (R2): logical row r (a RowJob row) is detector rows r * bin ..
    // r * bin + bin - 1 of raw_stride samples each (0: ixdim), sample x of the logical row the
    // truncated mean of the bin x bin block at columns raw_x0 + x * bin ..; bin <= 1: no binning
    long long raw_stride;
    int raw_x0;
    int bin;
    float lin16_scale;        // FP16 rows: the power-of-two scale of every row (fp16_row_scale)
};
cudaError_t launch_filter(const FilterLaunch& p, cudaStream_t s);
// The power-of-two scale that keeps every FP16 pair row of a filter table (ndim entries) below
// 16384 for any int16 sinogram: |r| <= 100 * 32768 * sqrt(sum_k H[k]^2), H[k] = (F[k] + F[-k]) / 2
// the filter's even part (the filtered row is a circular convolution of the placed row with a
// kernel whose L1 norm that bounds, by Cauchy-Schwarz and Parseval).
float fp16_row_scale(const float* filt, int ndim);
// 1 when kernels on the current device may read and write pageable host memory directly (the
// host's page tables are shared with the GPU, as on Grace-based systems); RV_NO_HOST_DIRECT=1
// turns the direct paths off
bool host_direct_access();
// dst (host or device) <- src (device), n bytes, by a kernel; both 16-byte aligned, n % 16 == 0
cudaError_t launch_copy16(void* dst, const void* src, size_t n, cudaStream_t s);

// ---- back-projection ---------------------------------------------------------------------
// LIN geometry of one view in FP64: detector coordinate u = x c + y s + off (zoomed pixels)
struct LinGeom {
    double c, s, off, pad;
};
struct BackprojLaunch {
    const int* table;         // REF: int tables, slot-major
    const void* rows16;       // LIN: pair rows (8 B FP32 or 4 B FP16 / BF16 per detector pixel)
    const float* row_scale;
    const float4* geom;       // per view {fcos, fsin, foffset, 0} (REF units: x16)
    const LinGeom* geom64;    // LIN: per view geometry in FP64 (slice stride geom_slice_stride)
    long long geom_slice_stride;  // float4s between the geometry of consecutive slices (0: shared)
    int nviews;               // views per slice
    int nslices;
    int ixdimp;
    long long table_stride;   // ints per view slot
    long long slice_table_stride;  // ints per slice (nviews * table_stride)
    long long row_stride;     // LIN: pairs per row
    long long slice_row_stride;
    void* out;                // int32 (REF) or float (LIN) slices, ixdimp^2 each
    long long out_slice_stride;  // elements per output slice
    int center_shift16;       // REF: 16 * integer centre offset added to foffset (R10)
    int mode;
    int table_fmt;            // REF table layout (must match the filter launch)
    unsigned int* status_counter;  // validation mode: window-violation counter (else null)
};
cudaError_t launch_backproject(const BackprojLaunch& p, cudaStream_t s);
// kernels launch_backproject started on this host thread since the previous call (then resets)
int take_backproject_launches();

// One tile of one slice for the persistent REF back-projection (batched queue).
struct TileJob {
    const int* table;         // the slice's tables (view-major, table_stride ints per view)
    const float4* geom;       // the slice's per-view geometry
    int* out;                 // the slice (ixdimp^2 int32)
    long long table_stride;
    int nviews, ixdimp, X0, Y0;
    int pair;                 // 1 or 2: also the next 1 or 2 slices (slice k's tables at table +
                              // k * nviews * table_stride, output at out + k * ixdimp^2), which
                              // share the geometry
    int accumulate;           // 1: add the tile's sums into out atomically (a group of views of
                              // the slice; out zeroed before), 0: store them
};
// tile shape of the persistent kernel of an int-table variant (0..4), and the default variant
void persistent_tile_xy(int variant, int* tx, int* ty);
int default_variant();
cudaError_t launch_bp_ref_persistent(const TileJob* d_jobs, int njobs, unsigned* d_counter, int table_fmt,
                                     int variant, cudaStream_t s);
cudaError_t launch_bp_ref(const BackprojLaunch& p, cudaStream_t s);
// the same with an explicit variant (0..20) instead of the process default
cudaError_t launch_bp_ref_variant(const BackprojLaunch& p, cudaStream_t s, int variant);
// LIN / FP16 / BF16 back-projection of pair rows (rows16 = pairs (r[j], r[j+1]-r[j]) of 8 or 4 bytes,
// row_stride / slice_row_stride in pairs, row_scale per row for the 16-bit forms)
cudaError_t launch_bp_lin(const BackprojLaunch& p, cudaStream_t s);
// pairs per stored LIN row (a multiple of 4 so every row starts on a 16-byte boundary)
inline int lin_pair_stride(int ixdimp) { return (ixdimp + 3) & ~3; }
inline int lin_pair_bytes(int mode) { return mode == RV_MODE_LIN ? 8 : 4; }
// REF table format per detector pixel j, and the slot stride in 4-byte words:
//   kTabInt16: the reference's 16 ints igp[16j+k]          (64 B per pixel)
//   kTabInt17: the same with one unused word after each 16  (68 B, fewer bank conflicts)
//   kTabPair:  the float pair (p0, p1p0) the 16 ints are made from (8 B); the back-projection
//              evaluates (int)(p0 + p1p0*k) itself with the reference's float operations
enum { kTabInt16 = 0, kTabInt17 = 1, kTabPair = 2 };
int ref_table_fmt();
long long ref_table_stride(int ixdimp, int fmt);
// fourth component of a REF view record {fcos, fsin, foffset, .}: the back-projection's ray-layout
// regime of the view, tagged (the kernels compute it themselves when the tag is absent)
float ray_regime_tag(float fcos, float fsin);
// Status word written by kernels whose bounded waits ran out (0 = fine); read-and-clear after
// synchronising stream s.  One word per device, shared by every call on it: a call whose work
// overlaps another's on the GPU may take the other's report.  kStatusUnreadable is returned
// when the word could not be read (a failed copy or synchronisation), never 0.
constexpr unsigned kStatusWaitRanOut = 1u;
constexpr unsigned kStatusUnreadable = 0x80000000u;
unsigned int take_kernel_status(cudaStream_t s);
const char* kernel_status_text(unsigned int status);

// ---- normalisation (R1) written back as int16 rows ------------------------------------------
struct NormLaunch {
    const uint16_t* raw;      // rows of the raw buffer (device), ixdim each
    short* out;               // destination rows (device), ixdim each
    const RowJob* jobs;       // src_row/flat/dark rows; dst = destination row
    int njobs;
    int ixdim;
    int pixmin;
    int zernike;
    const int* shift;         // per job drift shift in pixels (may be null)
    const uint16_t* const* row_ptr;  // if set: row r is row_ptr[r] for every role (it may be host
                                     // memory the device reads and writes directly), and the
                                     // result replaces row_ptr[dst] in place; raw/out unused
};
cudaError_t launch_normalise(const NormLaunch& p, cudaStream_t s);

int kernel_launches_per_filter();
}  // namespace rv
