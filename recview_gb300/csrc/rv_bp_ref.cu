// R8 (REF): back-projection with the reference's fixed-point 1/16 sub-sample table
// (source/general.cpp:2147-2158), bit-identical to the reference CPU routine.
//
// Work decomposition.  One CTA = a TX x TY pixel tile of one slice; a warp covers an 8x4 pixel
// block per register and each thread holds RX x RY int32 accumulators (pixels strided by the
// warp-grid extent).  Views are processed in chunks of VC.
//
// Table windows.  For each view a tile can only touch table entries between the projections of
// its corners.  Per chunk, one thread issues a TMA bulk copy (cp.async.bulk, completion on an
// mbarrier) of each view's window from the L2/HBM-resident table into shared memory, double
// buffered so chunk k+1 lands while chunk k is computed; parts of a window outside the table are
// zero-filled by the CTA, which implements the reference's range checks (ix0 < 0, ix0 >= 16 N)
// without a per-pixel branch.
//
// Per pixel and view:   fx  = fl(fl(ix*fcos) + fl(fl(iy*fsin) + foffset))      (tabulated terms)
//                       idx = (int)fx;   acc += igp[idx]
// (int)fx: when the corner bound shows fx >= 0 for the whole (tile, view), fl_rz(fx + 2^23) has
// the bit pattern 0x4B000000 + floor(fx) (exact for 0 <= fx < 2^23), so the index comes from the
// FP32 pipe and folds into the shared-memory address; otherwise cvt.rzi (F2I) keeps the
// reference's truncation of fx in (-1, 0) to entry 0.
//
// Window bound.  |computed fx - exact affine value| <= 2^-24 (|x fcos| + |y fsin| + 2 |fx|)
// < 0.1 for ixdimp <= 16384, and the affine value is extreme at the tile corners, so every
// index lies in [floor(min corner) - 1, floor(max corner) + 1]; the window spans
// [floor(min) - 2 (aligned down), floor(max) + 3).  The bounds-checked twin (CHECKED) counts any
// index outside the window; tests run it on many geometries and require zero.
//
// Optional padded layout (table_fmt): 17 words per detector pixel, so lanes whose indices differ
// by ~16 (views near 0 or 90 degrees) fall into different shared-memory banks.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "rv_internal.h"

namespace rv {

__device__ unsigned int g_kernel_status = 0;   // bit 0: an mbarrier wait ran out
// back-projection kernels launched on this host thread since take_backproject_launches()
static thread_local int t_bp_launches = 0;
static int env_int(const char* name, int dflt);  // tuning overrides from the environment

constexpr unsigned kMagicBits = 0x4B000000u;   // bit pattern of 2^23

__device__ __forceinline__ float fmulr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float faddr(float a, float b) { return __fadd_rn(a, b); }

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ int lds_s32(unsigned addr) {
    int v;
    asm volatile("ld.shared.s32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}
template <int OFF>
__device__ __forceinline__ int lds_s32_off(unsigned addr) {   // [addr + OFF], OFF in the instruction
    int v;
    asm volatile("ld.shared.s32 %0, [%1+%2];" : "=r"(v) : "r"(addr), "n"(OFF));
    return v;
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// One try: the thread may be suspended until the phase completes, for at most about the
// explicit suspend-time hint (1 us), so 2^20 tries bound a wait to about a second.
constexpr unsigned kTryWaitHintNs = 1000;
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "n"(kTryWaitHintNs)
        : "memory");
    return ok != 0;
}
// bounded wait: every spin has an iteration limit (2^LOG2 tries)
template <int LOG2 = 20>
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
    for (int i = 0; i < (1 << LOG2); i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_bulk_g2s(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

constexpr int isqrt_ceil(int n) {
    int r = 0;
    while (r * r < n) r++;
    return r;
}

template <int WX, int WY, int RX, int RY, int VC, int PAD, int OTF = 0>
struct BpCfg {
    static constexpr int NT = 32 * WX * WY;
    static constexpr int GX = 8 * WX, GY = 4 * WY;        // thread grid of the tile
    static constexpr int TX = GX * RX, TY = GY * RY;      // tile in pixels
    static constexpr int ALIGN = PAD ? 64 : 4;            // window start alignment (table index)
    // table-index span of a tile: 16*sqrt((TX-1)^2 + (TY-1)^2) + margins + alignment
    static constexpr int SPAN = 16 * isqrt_ceil((TX - 1) * (TX - 1) + (TY - 1) * (TY - 1)) + 2 + 3 + ALIGN + 16;
    static constexpr int WIN = PAD ? ((SPAN * 17 / 16 + 17 + 15) / 16) * 16 : ((SPAN + 15) / 16) * 16;
    // shared layout in words: windows [2][VC][WIN], tabulated products [3][VC][TX+TY] (absent
    // when OTF: the products are formed in registers), view records [3][VC][8], 2 mbarriers
    static constexpr int XY_WORDS = OTF ? 0 : 3 * VC * (TX + TY);
    static constexpr int META_OFF = 2 * VC * WIN + XY_WORDS;
    static constexpr int BAR_OFF = META_OFF + 3 * VC * 8;
    static constexpr size_t SMEM = (size_t)BAR_OFF * 4 + 16;
};

// Per-view record; the first 16 bytes are all the inner loop reads (one 128-bit load).
struct ViewMeta {
    float gc, gs, go;   // fcos, fsin, foffset of the view
    unsigned off;       // byte offset from the window base to entry 0 (bit 0: fast path)
    int w0;             // window start in table-storage words
    int nwin;           // window length in storage words (multiple of 4)
    int a, b;           // in-table part [a, b) of the window (storage words, multiples of 4)
};

// One tile of one slice.  ph[b] counts the completed phases of mbarrier b, so a persistent CTA
// can run many tiles on the same barriers.  Returns false when a bounded wait ran out.
// OTF = 1 forms the per-view column/row products in registers (12 FP32 operations per view per
// thread) instead of reading them from shared memory, which frees the shared-memory pipe -- the
// kernel's binding resource -- for the table gathers.  Both forms round identically.
template <int WX, int WY, int RX, int RY, int VC, int PAD, int OTF, bool CHECKED>
__device__ __forceinline__ bool bp_ref_tile(const TileJob& J, int* smi, unsigned (&ph)[2], unsigned* status_counter) {
    using Cfg = BpCfg<WX, WY, RX, RY, VC, PAD, OTF>;
    constexpr int NT = Cfg::NT, TX = Cfg::TX, TY = Cfg::TY, WIN = Cfg::WIN;
    int* win = smi;                                                     // [2][VC][WIN]
    float* xs = reinterpret_cast<float*>(win + 2 * VC * WIN);           // [3][VC][TX]   (OTF: unused)
    float* ys = xs + 3 * VC * TX;                                       // [3][VC][TY]
    ViewMeta* meta = reinterpret_cast<ViewMeta*>(smi + Cfg::META_OFF);  // [3][VC]
    uint64_t* bars = reinterpret_cast<uint64_t*>(smi + Cfg::BAR_OFF);   // [2]

    const int ixdimp = J.ixdimp;
    const int X0 = J.X0, Y0 = J.Y0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = (warp % WX) * 8 + (lane & 7);
    const int ty = (warp / WX) * 4 + (lane >> 3);
    const int* tab = J.table;
    const int nstore = PAD ? ((17 * ixdimp + 3) & ~3) : 16 * ixdimp;   // storage words per table row
    const int nviews = J.nviews;
    const int nchunks = (nviews + VC - 1) / VC;
    unsigned viol = 0;
    float colf[RX], rowf[RY];   // OTF: pixel coordinates as floats (exact: < 2^24)
#pragma unroll
    for (int c = 0; c < RX; c++) colf[c] = (float)(X0 + tx + Cfg::GX * c);
#pragma unroll
    for (int r = 0; r < RY; r++) rowf[r] = (float)(Y0 + ty + Cfg::GY * r);

    // window bounds (and, unless OTF, tabulated products) of chunk c into meta/xs/ys slot ms
    auto prepare = [&](int c, int ms) {
        const int v0 = c * VC;
        if (tid < VC && v0 + tid < nviews) {
            const float4 g = __ldg(J.geom + v0 + tid);
            float lo = 3.0e38f, hi = -3.0e38f;
#pragma unroll
            for (int cy = 0; cy < 2; cy++) {
                const float fy = faddr(fmulr((float)(Y0 + cy * (TY - 1)), g.y), g.z);
#pragma unroll
                for (int cx = 0; cx < 2; cx++) {
                    const float fx = faddr(fmulr((float)(X0 + cx * (TX - 1)), g.x), fy);
                    lo = fminf(lo, fx);
                    hi = fmaxf(hi, fx);
                }
            }
            const int ilo = (int)floorf(lo) - 2;
            const int lo_a = ilo >= 0 ? (ilo & ~(Cfg::ALIGN - 1)) : -((-ilo + Cfg::ALIGN - 1) & ~(Cfg::ALIGN - 1));
            const int ihi = (int)floorf(hi) + 3;   // exclusive
            ViewMeta m;
            if (PAD) {
                const int hi16 = (ihi + 15) & ~15;
                m.w0 = lo_a + lo_a / 16;              // 17 * lo_a / 16 (lo_a multiple of 64)
                const int w1 = hi16 + hi16 / 16;
                m.nwin = min(((w1 - m.w0) + 3) & ~3, WIN);
            } else {
                m.w0 = lo_a;
                m.nwin = min(((ihi - lo_a) + 3) & ~3, WIN);
            }
            m.a = max(m.w0, 0);
            m.b = min(m.w0 + m.nwin, nstore);
            const bool fast = lo >= 2.0f;
            m.gc = g.x;
            m.gs = g.y;
            m.go = g.z;
            // byte offset that turns the index bits into a shared-memory address (fast path: the
            // 2^23 pattern is folded in); unsigned wrap-around arithmetic, bit 0 flags the path
            const unsigned mag = PAD ? (kMagicBits + (kMagicBits >> 4)) : kMagicBits;
            m.off = (0u - 4u * (unsigned)m.w0 - (fast ? 4u * mag : 0u)) | (fast ? 1u : 0u);
            meta[ms * VC + tid] = m;
        }
        if (!OTF) {
            for (int e = tid; e < VC * (TX + TY); e += NT) {
                const int vv = e / (TX + TY), w = e - vv * (TX + TY);
                if (v0 + vv >= nviews) continue;
                const float4 g = __ldg(J.geom + v0 + vv);
                if (w < TX) {
                    const int t = w / RX, c = w - t * RX;          // xs[t*RX + c] = column of (tx=t, c)
                    xs[(ms * VC + vv) * TX + w] = fmulr((float)(X0 + t + Cfg::GX * c), g.x);
                } else {
                    const int w2 = w - TX, t = w2 / RY, r = w2 - t * RY;
                    ys[(ms * VC + vv) * TY + w2] = faddr(fmulr((float)(Y0 + t + Cfg::GY * r), g.y), g.z);
                }
            }
        }
    };
    // issue chunk c (meta slot ms) into window buffer wb: TMA by thread 0, zero-fill by all
    auto stage = [&](int c, int ms, int wb) {
        const int v0 = c * VC;
        const int nv = min(VC, nviews - v0);
        if (tid == 0) {
            unsigned bytes = 0;
            for (int vv = 0; vv < nv; vv++) {
                const ViewMeta m = meta[ms * VC + vv];
                if (m.b > m.a) bytes += 4u * (unsigned)(m.b - m.a);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const unsigned bar = smem_u32(&bars[wb]);
            mbar_arrive_expect_tx(bar, bytes);
            for (int vv = 0; vv < nv; vv++) {
                const ViewMeta m = meta[ms * VC + vv];
                if (m.b <= m.a) continue;
                const int* src = tab + (size_t)(v0 + vv) * J.table_stride + m.a;
                const unsigned dst = smem_u32(win + (wb * VC + vv) * WIN + (m.a - m.w0));
                tma_bulk_g2s(dst, src, 4u * (unsigned)(m.b - m.a), bar);
            }
        }
        for (int vv = 0; vv < nv; vv++) {
            const ViewMeta m = meta[ms * VC + vv];
            if (m.a == m.w0 && m.b == m.w0 + m.nwin) continue;   // inside the table: nothing to zero
            int4* w4 = reinterpret_cast<int4*>(win + (wb * VC + vv) * WIN);
            const int za = (m.b > m.a) ? (m.a - m.w0) >> 2 : m.nwin >> 2;   // [0, za) zero
            const int zb = (m.b > m.a) ? (m.b - m.w0) >> 2 : m.nwin >> 2;   // [zb, nwin) zero
            for (int e = tid; e < za; e += NT) w4[e] = make_int4(0, 0, 0, 0);
            for (int e = zb + tid; e < (m.nwin >> 2); e += NT) w4[e] = make_int4(0, 0, 0, 0);
        }
    };

    int acc[RY][RX];
#pragma unroll
    for (int r = 0; r < RY; r++)
#pragma unroll
        for (int c = 0; c < RX; c++) acc[r][c] = 0;

    prepare(0, 0);
    if (nchunks > 1) prepare(1, 1);
    __syncthreads();
    stage(0, 0, 0);

    for (int k = 0; k < nchunks; k++) {
        const int wb = k & 1, ms = k % 3;
        if (k + 1 < nchunks) stage(k + 1, (k + 1) % 3, wb ^ 1);
        if (k + 2 < nchunks) prepare(k + 2, (k + 2) % 3);
        const bool ok = mbar_wait_bounded(smem_u32(&bars[wb]), ph[wb] & 1u);
        if (__syncthreads_or(!ok)) {
            // a bulk copy did not complete in time: report, give the copies a bounded last
            // chance to land, and leave without touching the output
            if (tid == 0) atomicOr(&g_kernel_status, 1u);
            mbar_wait_bounded(smem_u32(&bars[wb]), ph[wb] & 1u);
            if (k + 1 < nchunks) mbar_wait_bounded(smem_u32(&bars[wb ^ 1]), ph[wb ^ 1] & 1u);
            return false;
        }
        ph[wb]++;
        const int nv = min(VC, nviews - k * VC);
        for (int vv = 0; vv < nv; vv++) {
            const float4 g = *reinterpret_cast<const float4*>(&meta[ms * VC + vv]);
            float xv[RX], yv[RY];
            if (OTF) {
#pragma unroll
                for (int c = 0; c < RX; c++) xv[c] = fmulr(colf[c], g.x);
#pragma unroll
                for (int r = 0; r < RY; r++) yv[r] = faddr(fmulr(rowf[r], g.y), g.z);
            } else {
#pragma unroll
                for (int c4 = 0; c4 < RX; c4 += 4) {
                    const float4 t4 = *reinterpret_cast<const float4*>(xs + (ms * VC + vv) * TX + tx * RX + c4);
                    xv[c4] = t4.x; xv[c4 + 1] = t4.y; xv[c4 + 2] = t4.z; xv[c4 + 3] = t4.w;
                }
#pragma unroll
                for (int r4 = 0; r4 < RY; r4 += 4) {
                    const float4 t4 = *reinterpret_cast<const float4*>(ys + (ms * VC + vv) * TY + ty * RY + r4);
                    yv[r4] = t4.x; yv[r4 + 1] = t4.y; yv[r4 + 2] = t4.z; yv[r4 + 3] = t4.w;
                }
            }
            const unsigned offb = __float_as_uint(g.w);
            const unsigned base = smem_u32(win + (wb * VC + vv) * WIN) + (offb & ~3u);
            int cw0 = 0, cnw = 0;
            if (CHECKED) {
                cw0 = meta[ms * VC + vv].w0;
                cnw = meta[ms * VC + vv].nwin;
            }
            if (offb & 1u) {
                // index v = bits - 2^23 pattern; PAD: storage = v + (v >> 4)
#pragma unroll
                for (int r = 0; r < RY; r++)
#pragma unroll
                    for (int c = 0; c < RX; c++) {
                        const float fx = faddr(xv[c], yv[r]);
                        const unsigned bits = __float_as_uint(__fadd_rz(fx, 8388608.0f));
                        const unsigned st = PAD ? bits + (bits >> 4) : bits;
                        if (CHECKED) {
                            const int v = (int)(bits - kMagicBits);
                            const int sw = PAD ? v + (v >> 4) : v;
                            if (fx < 0.0f || sw < cw0 || sw >= cw0 + cnw) { viol++; continue; }
                        }
                        acc[r][c] += lds_s32(base + 4u * st);
                    }
            } else {
#pragma unroll
                for (int r = 0; r < RY; r++)
#pragma unroll
                    for (int c = 0; c < RX; c++) {
                        const float fx = faddr(xv[c], yv[r]);
                        const int v = __float2int_rz(fx);
                        const int sw = PAD ? v + (v >> 4) : v;
                        if (CHECKED) {
                            if (sw < cw0 || sw >= cw0 + cnw) { viol++; continue; }
                        }
                        acc[r][c] += lds_s32(base + 4u * (unsigned)sw);
                    }
            }
        }
        __syncthreads();
    }
    if (CHECKED && viol) atomicAdd(status_counter, viol);

    int* out = J.out;
#pragma unroll
    for (int r = 0; r < RY; r++) {
        const int y = Y0 + ty + Cfg::GY * r;
        if (y >= ixdimp) continue;
#pragma unroll
        for (int c = 0; c < RX; c++) {
            const int x = X0 + tx + Cfg::GX * c;
            if (x < ixdimp) out[(size_t)y * ixdimp + x] = acc[r][c];
        }
    }
    __syncthreads();   // the next tile of a persistent CTA reuses the shared buffers
    return true;
}

template <int WX, int WY, int RX, int RY, int VC, int PAD, int OTF>
__device__ __forceinline__ void bp_init_barriers(int* smi) {
    using Cfg = BpCfg<WX, WY, RX, RY, VC, PAD, OTF>;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smi + Cfg::BAR_OFF);
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bars[0]), 1);
        mbar_init(smem_u32(&bars[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

// Grid form: blockIdx.x = tile, blockIdx.y = slice.
template <int WX, int WY, int RX, int RY, int VC, int PAD, int MINB, int OTF, bool CHECKED>
__global__ void __launch_bounds__(32 * WX * WY, MINB) k_bp_ref(BackprojLaunch p) {
    using Cfg = BpCfg<WX, WY, RX, RY, VC, PAD, OTF>;
    extern __shared__ __align__(128) int smi[];
    bp_init_barriers<WX, WY, RX, RY, VC, PAD, OTF>(smi);
    const int tiles_x = (p.ixdimp + Cfg::TX - 1) / Cfg::TX;
    TileJob J;
    J.table = p.table + (size_t)blockIdx.y * p.slice_table_stride;
    J.geom = p.geom + (size_t)blockIdx.y * p.geom_slice_stride;
    J.out = static_cast<int*>(p.out) + (size_t)blockIdx.y * p.out_slice_stride;
    J.table_stride = p.table_stride;
    J.nviews = p.nviews;
    J.ixdimp = p.ixdimp;
    J.X0 = (blockIdx.x % tiles_x) * Cfg::TX;
    J.Y0 = (blockIdx.x / tiles_x) * Cfg::TY;
    unsigned ph[2] = {0u, 0u};
    bp_ref_tile<WX, WY, RX, RY, VC, PAD, OTF, CHECKED>(J, smi, ph, p.status_counter);
}

// Persistent form: each CTA takes tiles from a device work list (uneven datasets) until it is
// exhausted; *counter must be zero at launch.
template <int WX, int WY, int RX, int RY, int VC, int PAD, int MINB, int OTF>
__global__ void __launch_bounds__(32 * WX * WY, MINB) k_bp_ref_persistent(const TileJob* jobs, int njobs,
                                                                          unsigned* counter) {
    extern __shared__ __align__(128) int smi[];
    __shared__ int s_item;
    bp_init_barriers<WX, WY, RX, RY, VC, PAD, OTF>(smi);
    unsigned ph[2] = {0u, 0u};
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= njobs) break;
        if (!bp_ref_tile<WX, WY, RX, RY, VC, PAD, OTF, false>(jobs[it], smi, ph, nullptr)) return;
    }
}

// ---- warp-decoupled pipeline ------------------------------------------------------------------
// The same per-update arithmetic as bp_ref_tile (products in registers), but without a block-wide
// barrier per chunk: NB window buffers, each with a "full" mbarrier (completed by the TMA bytes)
// and an "empty" mbarrier (one arrival per warp when it has finished reading the buffer).  Warp 0
// also produces: before consuming chunk c it refills the buffer of chunk c-1 with chunk c+NB-1,
// after that buffer's empty barrier shows every warp is done with it.  Other warps never wait
// for each other, only for data.  Every wait is bounded; a timeout sets g_kernel_status, gives
// the copies this CTA issued a bounded chance to land, and ends the tile.
template <int WX, int WY, int RX, int RY, int VC, int NB, int PAD>
struct PipeCfg {
    using Base = BpCfg<WX, WY, RX, RY, VC, PAD, 1>;
    static constexpr int NT = Base::NT, NW = NT / 32;
    static constexpr int GX = Base::GX, GY = Base::GY, TX = Base::TX, TY = Base::TY;
    static constexpr int ALIGN = Base::ALIGN, WIN = Base::WIN;
    static constexpr int META_OFF = NB * VC * WIN;             // words
    static constexpr int BAR_OFF = META_OFF + NB * VC * 8;     // full[NB], empty[NB] (8 B each)
    static constexpr size_t SMEM = (size_t)BAR_OFF * 4 + (size_t)2 * NB * 8;
};

template <int WX, int WY, int RX, int RY, int VC, int NB, int PAD>
__device__ __forceinline__ void pipe_init_barriers(int* smi) {
    using Cfg = PipeCfg<WX, WY, RX, RY, VC, NB, PAD>;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smi + Cfg::BAR_OFF);
    if (threadIdx.x == 0) {
        for (int b = 0; b < NB; b++) {
            mbar_init(smem_u32(&bars[b]), 1);
            mbar_init(smem_u32(&bars[NB + b]), Cfg::NW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

// The record of one view for a TX x TY tile at (X0, Y0): geometry, the table window the tile can
// touch (start aligned to ALIGN, length a multiple of 4 words, at most WIN), the in-table part of
// that window (nstore = table words per view slot) and the fast-path byte offset.
template <int TX, int TY, int WIN, int ALIGN, int PAD>
__device__ __forceinline__ ViewMeta view_window(float4 gg, int X0, int Y0, int nstore) {
    float lo = 3.0e38f, hi = -3.0e38f;
#pragma unroll
    for (int cy = 0; cy < 2; cy++) {
        const float fy = faddr(fmulr((float)(Y0 + cy * (TY - 1)), gg.y), gg.z);
#pragma unroll
        for (int cx = 0; cx < 2; cx++) {
            const float fx = faddr(fmulr((float)(X0 + cx * (TX - 1)), gg.x), fy);
            lo = fminf(lo, fx);
            hi = fmaxf(hi, fx);
        }
    }
    const int ilo = (int)floorf(lo) - 2;
    const int lo_a = ilo >= 0 ? (ilo & ~(ALIGN - 1)) : -((-ilo + ALIGN - 1) & ~(ALIGN - 1));
    const int ihi = (int)floorf(hi) + 3;
    ViewMeta m;
    if (PAD) {
        const int hi16 = (ihi + 15) & ~15;
        m.w0 = lo_a + lo_a / 16;
        const int w1 = hi16 + hi16 / 16;
        m.nwin = min(((w1 - m.w0) + 3) & ~3, WIN);
    } else {
        m.w0 = lo_a;
        m.nwin = min(((ihi - lo_a) + 3) & ~3, WIN);
    }
    m.a = max(m.w0, 0);
    m.b = min(m.w0 + m.nwin, nstore);
    const bool fast = lo >= 2.0f;
    m.gc = gg.x;
    m.gs = gg.y;
    m.go = gg.z;
    const unsigned mag = PAD ? (kMagicBits + (kMagicBits >> 4)) : kMagicBits;
    m.off = (0u - 4u * (unsigned)m.w0 - (fast ? 4u * mag : 0u)) | (fast ? 1u : 0u);
    return m;
}

// Warp 0 of a pipelined CTA: fill buffer g % NB with the table windows of chunk c (views
// c*VC ..) once that buffer's empty barrier shows every warp is done with it.  Records each view's
// geometry and window in meta, zero-fills the parts of a window outside the table, and issues one
// TMA bulk copy per view on the buffer's full barrier.  Returns false (warp-uniform) when the wait
// for the empty barrier ran out.
// NS = 2 stages, for every view, the windows of two slices that share the geometry (the same
// window bounds, tables J.table + s * slice_tab_stride) one after the other: window (b, vv, s) at
// ((b * VC + vv) * NS + s) * WIN.
// NSL (>= NS) is the number of window slots per view in the buffer layout.
template <int TX, int TY, int WIN, int ALIGN, int VC, int NB, int PAD, int NS = 1, int NSL = NS>
__device__ __forceinline__ bool pipe_fill(const TileJob& J, int* win, ViewMeta* meta, uint64_t* bars, int c,
                                          unsigned g, int lane, long long slice_tab_stride = 0) {
    const int X0 = J.X0, Y0 = J.Y0;
    const int nviews = J.nviews;
    const int nstore = PAD ? ((17 * J.ixdimp + 3) & ~3) : 16 * J.ixdimp;
    const int b = (int)(g % NB);
    // warp-uniform verdict: every lane takes the same branch at the __syncwarp()s below
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[NB + b]), ((g / NB) & 1u) ^ 1u)))
        return false;
    const int v0 = c * VC;
    const int nv = min(VC, nviews - v0);
    if (lane < nv) meta[b * VC + lane] = view_window<TX, TY, WIN, ALIGN, PAD>(__ldg(J.geom + v0 + lane), X0, Y0, nstore);
    __syncwarp();
    for (int vv = 0; vv < nv; vv++) {
        const ViewMeta m = meta[b * VC + vv];
        if (m.a == m.w0 && m.b == m.w0 + m.nwin) continue;
        const int za = (m.b > m.a) ? (m.a - m.w0) >> 2 : m.nwin >> 2;
        const int zb = (m.b > m.a) ? (m.b - m.w0) >> 2 : m.nwin >> 2;
#pragma unroll
        for (int sl = 0; sl < NS; sl++) {
            int4* w4 = reinterpret_cast<int4*>(win + ((b * VC + vv) * NSL + sl) * WIN);
            for (int e = lane; e < za; e += 32) w4[e] = make_int4(0, 0, 0, 0);
            for (int e = zb + lane; e < (m.nwin >> 2); e += 32) w4[e] = make_int4(0, 0, 0, 0);
        }
    }
    __syncwarp();
    if (lane == 0) {
        unsigned bytes = 0;
        for (int vv = 0; vv < nv; vv++) {
            const ViewMeta m = meta[b * VC + vv];
            if (m.b > m.a) bytes += 4u * NS * (unsigned)(m.b - m.a);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const unsigned bar = smem_u32(&bars[b]);
        mbar_arrive_expect_tx(bar, bytes);
        for (int vv = 0; vv < nv; vv++) {
            const ViewMeta m = meta[b * VC + vv];
            if (m.b <= m.a) continue;
#pragma unroll
            for (int sl = 0; sl < NS; sl++) {
                const int* src = J.table + sl * slice_tab_stride + (size_t)(v0 + vv) * J.table_stride + m.a;
                const unsigned dst = smem_u32(win + ((b * VC + vv) * NSL + sl) * WIN + (m.a - m.w0));
                tma_bulk_g2s(dst, src, 4u * (unsigned)(m.b - m.a), bar);
            }
        }
    }
    __syncwarp();
    return true;
}

// One tile.  gc = chunks this CTA has run through the buffers before this tile (the phase
// bookkeeping of a persistent CTA); returns false after a bounded wait ran out.
template <int WX, int WY, int RX, int RY, int VC, int NB, int PAD, bool CHECKED>
__device__ __forceinline__ bool bp_ref_tile_pipe(const TileJob& J, int* smi, unsigned gc, unsigned* status_counter) {
    using Cfg = PipeCfg<WX, WY, RX, RY, VC, NB, PAD>;
    constexpr int TX = Cfg::TX, TY = Cfg::TY, WIN = Cfg::WIN;
    int* win = smi;                                                     // [NB][VC][WIN]
    ViewMeta* meta = reinterpret_cast<ViewMeta*>(smi + Cfg::META_OFF);  // [NB][VC]
    uint64_t* bars = reinterpret_cast<uint64_t*>(smi + Cfg::BAR_OFF);   // full[NB], empty[NB]
    const int ixdimp = J.ixdimp;
    const int X0 = J.X0, Y0 = J.Y0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = (warp % WX) * 8 + (lane & 7);
    const int ty = (warp / WX) * 4 + (lane >> 3);
    const int nviews = J.nviews;
    const int nchunks = (nviews + VC - 1) / VC;
    unsigned viol = 0;
    float colf[RX], rowf[RY];
#pragma unroll
    for (int c = 0; c < RX; c++) colf[c] = (float)(X0 + tx + Cfg::GX * c);
#pragma unroll
    for (int r = 0; r < RY; r++) rowf[r] = (float)(Y0 + ty + Cfg::GY * r);

    // warp 0: fill the buffer of chunk c (global chunk number g); false on a timeout
    auto produce = [&](int c, unsigned g) -> bool {
        return pipe_fill<TX, TY, WIN, Cfg::ALIGN, VC, NB, PAD>(J, win, meta, bars, c, g, lane);
    };

    int acc[RY][RX];
#pragma unroll
    for (int r = 0; r < RY; r++)
#pragma unroll
        for (int c = 0; c < RX; c++) acc[r][c] = 0;

    bool ok = true;
    int produced = 0;   // warp 0: chunks of this tile whose fill has been issued
    if (warp == 0) {
        for (; produced < nchunks && produced < NB - 1; produced++)
            if (!produce(produced, gc + (unsigned)produced)) { ok = false; break; }
    }
    for (int k = 0; ok && k < nchunks; k++) {
        if (warp == 0 && produced < nchunks) {
            if (!produce(produced, gc + (unsigned)produced)) { ok = false; break; }
            produced++;
        }
        const unsigned g = gc + (unsigned)k;
        const int b = (int)(g % NB);
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[b]), (g / NB) & 1u))) { ok = false; break; }
        const int nv = min(VC, nviews - k * VC);
        for (int vv = 0; vv < nv; vv++) {
            const float4 gm = *reinterpret_cast<const float4*>(&meta[b * VC + vv]);
            float xv[RX], yv[RY];
#pragma unroll
            for (int c = 0; c < RX; c++) xv[c] = fmulr(colf[c], gm.x);
#pragma unroll
            for (int r = 0; r < RY; r++) yv[r] = faddr(fmulr(rowf[r], gm.y), gm.z);
            const unsigned offb = __float_as_uint(gm.w);
            const unsigned base = smem_u32(win + (b * VC + vv) * WIN) + (offb & ~3u);
            int cw0 = 0, cnw = 0;
            if (CHECKED) {
                cw0 = meta[b * VC + vv].w0;
                cnw = meta[b * VC + vv].nwin;
            }
            if (offb & 1u) {
#pragma unroll
                for (int r = 0; r < RY; r++)
#pragma unroll
                    for (int c = 0; c < RX; c++) {
                        const float fx = faddr(xv[c], yv[r]);
                        const unsigned bits = __float_as_uint(__fadd_rz(fx, 8388608.0f));
                        const unsigned st = PAD ? bits + (bits >> 4) : bits;
                        if (CHECKED) {
                            const int v = (int)(bits - kMagicBits);
                            const int sw = PAD ? v + (v >> 4) : v;
                            if (fx < 0.0f || sw < cw0 || sw >= cw0 + cnw) { viol++; continue; }
                        }
                        acc[r][c] += lds_s32(base + 4u * st);
                    }
            } else {
#pragma unroll
                for (int r = 0; r < RY; r++)
#pragma unroll
                    for (int c = 0; c < RX; c++) {
                        const float fx = faddr(xv[c], yv[r]);
                        const int v = __float2int_rz(fx);
                        const int sw = PAD ? v + (v >> 4) : v;
                        if (CHECKED) {
                            if (sw < cw0 || sw >= cw0 + cnw) { viol++; continue; }
                        }
                        acc[r][c] += lds_s32(base + 4u * (unsigned)sw);
                    }
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&bars[NB + b]));
    }
    if (!ok) {
        atomicOr(&g_kernel_status, 1u);
        // warp 0 issued fills up to chunk `produced`: give them a bounded chance to land before
        // the CTA can leave (later consumers of these buffers are gone)
        if (warp == 0) {
            for (int c = produced > NB ? produced - NB : 0; c < produced; c++) {   // last fill of each buffer
                const unsigned g = gc + (unsigned)c;
                mbar_wait_bounded(smem_u32(&bars[g % NB]), (g / NB) & 1u);
            }
        }
        return false;
    }
    if (CHECKED && viol) atomicAdd(status_counter, viol);
    int* out = J.out;
#pragma unroll
    for (int r = 0; r < RY; r++) {
        const int y = Y0 + ty + Cfg::GY * r;
        if (y >= ixdimp) continue;
#pragma unroll
        for (int c = 0; c < RX; c++) {
            const int x = X0 + tx + Cfg::GX * c;
            if (x < ixdimp) out[(size_t)y * ixdimp + x] = acc[r][c];
        }
    }
    return true;
}

template <int WX, int WY, int RX, int RY, int VC, int NB, int PAD, int MINB, bool CHECKED>
__global__ void __launch_bounds__(32 * WX * WY, MINB) k_bp_ref_pipe(BackprojLaunch p) {
    using Cfg = PipeCfg<WX, WY, RX, RY, VC, NB, PAD>;
    extern __shared__ __align__(128) int smi[];
    pipe_init_barriers<WX, WY, RX, RY, VC, NB, PAD>(smi);
    __syncthreads();
    const int tiles_x = (p.ixdimp + Cfg::TX - 1) / Cfg::TX;
    TileJob J;
    J.table = p.table + (size_t)blockIdx.y * p.slice_table_stride;
    J.geom = p.geom + (size_t)blockIdx.y * p.geom_slice_stride;
    J.out = static_cast<int*>(p.out) + (size_t)blockIdx.y * p.out_slice_stride;
    J.table_stride = p.table_stride;
    J.nviews = p.nviews;
    J.ixdimp = p.ixdimp;
    J.X0 = (blockIdx.x % tiles_x) * Cfg::TX;
    J.Y0 = (blockIdx.x / tiles_x) * Cfg::TY;
    bp_ref_tile_pipe<WX, WY, RX, RY, VC, NB, PAD, CHECKED>(J, smi, 0u, p.status_counter);
}

template <int WX, int WY, int RX, int RY, int VC, int NB, int PAD, int MINB>
__global__ void __launch_bounds__(32 * WX * WY, MINB) k_bp_ref_pipe_persistent(const TileJob* jobs, int njobs,
                                                                               unsigned* counter) {
    extern __shared__ __align__(128) int smi[];
    __shared__ int s_item;
    pipe_init_barriers<WX, WY, RX, RY, VC, NB, PAD>(smi);
    unsigned gc = 0;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= njobs) break;
        const TileJob J = jobs[it];
        const bool tok = bp_ref_tile_pipe<WX, WY, RX, RY, VC, NB, PAD, false>(J, smi, gc, nullptr);
        if (__syncthreads_or(!tok)) return;   // the CTA leaves together after a timeout
        gc += (unsigned)((J.nviews + VC - 1) / VC);
    }
}

// ---- warp-specialised producer, ray-aligned lane footprints ------------------------------------
// Changes to the warp-decoupled pipeline above, each bit-identical.
//
// Producer warp.  One extra warp only fills window buffers: it waits for a buffer's empty
// barrier, records the views' windows and issues their TMA copies, so the CW consumer warps never
// wait for a fill that a busy consumer has not issued yet, and all of them do the same work.
//
// Ray-aligned footprints (NQ > 0).  A warp's 32 lookups of one view cost one shared-memory
// wavefront per distinct word in its busiest bank.  A compact 8x4 pixel block spreads the lanes'
// indices over ~100 words (2.3 wavefronts per gather).  Here every register of a warp holds 32
// pixels along one line of the view's iso-index direction (x*fcos + y*fsin = const), so its
// indices fall within a few dozen consecutive words (~1.3 wavefronts).
// Layouts: a 64x64 tile, CW consumer warps (8 or 16), Q = 64 / CW sheared coordinates per thread,
// 2Q accumulators per thread and slice in slots s = 2q + p (q < Q, p 0..1); w = warp, j = lane.
// A regime is an orientation and a shear k in [-NQ, NQ]:
//     V (|fcos| >= |fsin|):  x = (w + sh(j) + CW q) mod 64,  y = j + 32p,   sh(j) = round(j k / NQ)
//     H (|fsin| >  |fcos|):  x = j + 32p,  y = (w + sh(j) + CW q) mod 64
// Each maps (w, j, q, p) one-to-one onto the tile, and a thread's pixels are Q sheared x 2 fixed
// coordinates, so the per-view products cost Q + 2*2 (V) or 2 + 2Q (H) FP32 operations.
// The regime of a chunk follows from the geometry of its first view (every consumer computes
// the same value).  When it changes, the accumulators move through the buffer just consumed,
// between barriers of the consumer warps: written at (slot, thread), read back from the old owner
// of each new pixel.  Two layouts of the same orientation give each pixel the same lane in both,
// so that exchange is free of bank conflicts.  Every pixel still sums the same int32 entries over
// the same views.
//
// Slice pairs (NS = 2).  Two slices that share the geometry share every index: a pixel's second
// gather is one more shared load at a fixed offset (the second slice's window follows the first)
// and one more add.
//
// Failure protocol.  The consumer barriers of an exchange need all consumer warps, so a warp
// whose bounded wait ran out does not leave the loop: it raises the CTA's abort word (the others
// then skip their waits), skips the rest of its work, and the consumers leave together at the
// next exchange or after the last chunk; the producer stops at the abort word or at its own
// bounded wait.  All threads then meet at one block barrier.
template <int CW>
__device__ __forceinline__ bool consumers_bar_or(bool pred) {   // named barrier 1: the consumers
    unsigned r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, %2, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((unsigned)pred), "n"(32 * CW)
        : "memory");
    return r != 0;
}
template <int CW>
__device__ __forceinline__ void consumers_bar() {
    asm volatile("bar.sync 1, %0;" ::"n"(32 * CW) : "memory");
}

// The producer warp of a warp-specialised CTA: publish chunk c's view records m (lane vv holds
// view vv's, computed before this call) in buffer g % NB once its empty barrier shows every
// consumer is done with it, zero-fill the window parts outside the table (edge tiles only), and
// issue the bulk copies -- lane vv those of view vv -- on the buffer's full barrier.  Only the
// record stores and the copy issue remain after the empty barrier; the geometry loads and the
// window arithmetic of the next chunk run while the consumers still read the buffer.  Returns
// false (warp-uniform) when the bounded wait ran out.
template <int WIN, int VC, int NB, int NS, int NSL>
__device__ __forceinline__ bool ws_fill(const TileJob& J, int* win, ViewMeta* meta, uint64_t* bars, int v0, int nv,
                                        unsigned g, int lane, const ViewMeta& m, long long slice_tab_stride) {
    const int b = (int)(g % NB);
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[NB + b]), ((g / NB) & 1u) ^ 1u)))
        return false;
    const bool mine = lane < nv;
    if (mine) meta[b * VC + lane] = m;
    unsigned edges = __ballot_sync(0xffffffffu, mine && !(m.a == m.w0 && m.b == m.w0 + m.nwin));
    while (edges) {   // warp-uniform
        const int vv = __ffs(edges) - 1;
        edges &= edges - 1;
        const int w0 = __shfl_sync(0xffffffffu, m.w0, vv), nwin = __shfl_sync(0xffffffffu, m.nwin, vv);
        const int a = __shfl_sync(0xffffffffu, m.a, vv), e1 = __shfl_sync(0xffffffffu, m.b, vv);
        const int za = (e1 > a) ? (a - w0) >> 2 : nwin >> 2;
        const int zb = (e1 > a) ? (e1 - w0) >> 2 : nwin >> 2;
#pragma unroll
        for (int sl = 0; sl < NS; sl++) {
            int4* w4 = reinterpret_cast<int4*>(win + ((b * VC + vv) * NSL + sl) * WIN);
            for (int e = lane; e < za; e += 32) w4[e] = make_int4(0, 0, 0, 0);
            for (int e = zb + lane; e < (nwin >> 2); e += 32) w4[e] = make_int4(0, 0, 0, 0);
        }
    }
    const bool copy = mine && m.b > m.a;
    const unsigned bytes = __reduce_add_sync(0xffffffffu, copy ? 4u * NS * (unsigned)(m.b - m.a) : 0u);
    // the records and zero fills are ordered before the barrier's completion, and every
    // lane's generic accesses to the buffer before its own copies into it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncwarp();
    const unsigned bar = smem_u32(&bars[b]);
    if (lane == 0) mbar_arrive_expect_tx(bar, bytes);
    __syncwarp();
    if (copy) {
#pragma unroll
        for (int sl = 0; sl < NS; sl++) {
            const int* src = J.table + sl * slice_tab_stride + (size_t)(v0 + lane) * J.table_stride + m.a;
            const unsigned dst = smem_u32(win + ((b * VC + lane) * NSL + sl) * WIN + (m.a - m.w0));
            tma_bulk_g2s(dst, src, 4u * (unsigned)(m.b - m.a), bar);
        }
    }
    return true;
}

template <int VC, int NB, int PAD, int NS = 1, int CW = 8>
struct WsCfg {
    using Pipe = PipeCfg<2, 4, 4, 4, VC, NB, PAD>;   // 64x64 tile: the same window size
    static constexpr int NT = 32 * CW + 32;          // CW consumer warps + 1 producer warp
    static constexpr int Q = 64 / CW, S = 2 * Q;     // sheared coordinates and pixels per thread
    static constexpr int TX = Pipe::TX, TY = Pipe::TY, ALIGN = Pipe::ALIGN, WIN = Pipe::WIN;
    static constexpr int META_OFF = NB * VC * NS * WIN;      // words: windows [NB][VC][NS][WIN]
    static constexpr int BAR_OFF = META_OFF + NB * VC * 8;   // view records [NB][VC]
    static constexpr int ABORT_OFF = BAR_OFF + 4 * NB;       // after full[NB], empty[NB]
    static constexpr size_t SMEM = (size_t)ABORT_OFF * 4 + 16;
    static constexpr bool EXCHANGE_FITS = VC * NS * WIN >= 4096;   // one buffer holds a slice's exchange
    static_assert(TX == 64 && TY == 64 && (CW == 8 || CW == 16), "8 or 16 consumer warps tile 64x64 pixels");
};

// regime = orientation (bit 0: H) | (k + NQ) << 1, from a view's fcos, fsin; any value gives the
// same slice, it only has to be the same in every consumer thread (a pure function of the inputs)
template <int NQ>
__device__ __forceinline__ int ray_regime(float gc, float gs) {
    const bool h = fabsf(gs) > fabsf(gc);
    const float t = h ? __fdividef(-gc, gs) : __fdividef(-gs, gc);   // |t| <= 1
    int k = __float2int_rn(t * (float)NQ);                             // NaN (fcos = fsin = 0) gives 0
    k = max(-NQ, min(NQ, k));
    return (h ? 1 : 0) | ((k + NQ) << 1);
}
// The regime of a view record: the producer of the geometry may store it in the record's unused
// fourth component, tagged with NQ (ray_regime_tag, host side); otherwise it is computed here.
constexpr unsigned kRegimeTag = 0x52000000u;   // | NQ << 16 | regime
template <int NQ>
__device__ __forceinline__ int regime_of(float4 g) {
    const unsigned w = __float_as_uint(g.w);
    if ((w >> 16) == ((kRegimeTag >> 16) | (unsigned)NQ)) return (int)(w & 0xffffu);
    return ray_regime<NQ>(g.x, g.y);
}
// sh(j) = round(j k / NQ), halves up (the numerator is kept positive for the division)
template <int NQ>
__device__ __forceinline__ int ray_shift(int j, int regime) {
    constexpr int D = NQ > 0 ? 2 * NQ : 1;   // (NQ = 0, the compact layout, never shears)
    const int k = (regime >> 1) - NQ;
    return NQ > 0 ? (2 * j * k + NQ + 128 * NQ) / D - 64 : 0;
}
// the thread's sheared (lin) and fixed (fix) absolute pixel coordinates under a regime
template <int NQ, int CW>
__device__ __forceinline__ void ray_coords(int regime, int X0, int Y0, int warp, int lane, float (&lin)[64 / CW],
                                           float (&fix)[2]) {
    const int sh = ray_shift<NQ>(lane, regime);
    const int lb = (regime & 1) ? Y0 : X0, fb = (regime & 1) ? X0 : Y0;
#pragma unroll
    for (int q = 0; q < 64 / CW; q++) lin[q] = (float)(lb + ((warp + sh + CW * q) & 63));
#pragma unroll
    for (int p = 0; p < 2; p++) fix[p] = (float)(fb + lane + 32 * p);
}

__device__ __forceinline__ float2 bcast2(float v) { return make_float2(v, v); }
// Paired FP32 additions (two lanes per instruction), each lane rounded like the scalar addition.
// Only additions are paired: the compiler fuses a paired multiply into a following paired add
// (one rounding instead of two) even with explicit rounding, so every product is a scalar
// __fmul_rn, which it never fuses.
__device__ __forceinline__ unsigned long long pk2(float2 v) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}
__device__ __forceinline__ float2 upk2(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
__device__ __forceinline__ float2 add2_rz(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk2(a)), "l"(pk2(b)));
    return upk2(d);
}

// slot of half h of slot pair i.  Ray layouts: slot 2q + p, pairs (q, q+1) at even q;
// compact (8 consumer warps): slot 4r + c, pairs (c, c+1)
template <bool COMPACT>
__device__ __forceinline__ constexpr int ws_slot(int i, int h) {
    return COMPACT ? 4 * (i >> 1) + 2 * (i & 1) + h : 4 * (i >> 1) + (i & 1) + 2 * h;
}
// acc[sl][s] += the entry at byte address a of slice sl's window (the NS windows of a view follow
// each other WIN words apart, so every slice after the first is one load with a fixed offset)
template <int NS, int WIN, int S>
__device__ __forceinline__ void ws_add_slices(int (&acc)[NS][S], int s, unsigned a) {
    acc[0][s] += lds_s32(a);
    if (NS > 1) acc[1 % NS][s] += lds_s32_off<4 * WIN * (NS > 1 ? 1 : 0)>(a);
    if (NS > 2) acc[2 % NS][s] += lds_s32_off<4 * WIN * (NS > 2 ? 2 : 0)>(a);
    if (NS > 3) acc[3 % NS][s] += lds_s32_off<4 * WIN * (NS > 3 ? 3 : 0)>(a);
}
// acc[sl][s] += the table entry of slot s's pixel in slice sl, for one view of a staged chunk.
// fx2(i) gives fl(fl(x fcos) + fl(fl(y fsin) + foffset)) of the two pixels of slot pair i.
template <int VC, int WIN, int PAD, bool CHECKED, int NS, int NSL, bool COMPACT, int S, typename FX2>
__device__ __forceinline__ void ws_gather(int (&acc)[NS][S], const int* win, const ViewMeta* meta, int b, int vv,
                                          unsigned offb, unsigned& viol, FX2 fx2) {
    const unsigned base = smem_u32(win + (b * VC + vv) * NSL * WIN) + (offb & ~3u);
    int cw0 = 0, cnw = 0;
    if (CHECKED) {
        cw0 = meta[b * VC + vv].w0;
        cnw = meta[b * VC + vv].nwin;
    }
    if (offb & 1u) {
        const float2 mag = make_float2(8388608.0f, 8388608.0f);
#pragma unroll
        for (int i = 0; i < S / 2; i++) {
            const float2 fx = fx2(i);
            const float2 t = add2_rz(fx, mag);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int s = ws_slot<COMPACT>(i, h);
                const unsigned bits = __float_as_uint(h ? t.y : t.x);
                const unsigned st = PAD ? bits + (bits >> 4) : bits;
                if (CHECKED) {
                    const int v = (int)(bits - kMagicBits);
                    const int sw = PAD ? v + (v >> 4) : v;
                    if ((h ? fx.y : fx.x) < 0.0f || sw < cw0 || sw >= cw0 + cnw) { viol++; continue; }
                }
                ws_add_slices<NS, WIN>(acc, s, base + 4u * st);
            }
        }
    } else {
#pragma unroll
        for (int i = 0; i < S / 2; i++) {
            const float2 fx = fx2(i);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int s = ws_slot<COMPACT>(i, h);
                const int v = __float2int_rz(h ? fx.y : fx.x);
                const int sw = PAD ? v + (v >> 4) : v;
                if (CHECKED) {
                    if (sw < cw0 || sw >= cw0 + cnw) { viol++; continue; }
                }
                ws_add_slices<NS, WIN>(acc, s, base + 4u * (unsigned)sw);
            }
        }
    }
}

// Two views at once (both on the fast path): each pixel's two gathers are added in one
// three-operand integer add.
template <int WIN, int PAD, int NS, int S, typename FA, typename FB>
__device__ __forceinline__ void ws_gather_two(int (&acc)[NS][S], unsigned baseA, unsigned baseB, FA fa, FB fb) {
    const float2 mag = make_float2(8388608.0f, 8388608.0f);
#pragma unroll
    for (int i = 0; i < S / 2; i++) {
        const float2 tA = add2_rz(fa(i), mag), tB = add2_rz(fb(i), mag);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int s = ws_slot<false>(i, h);
            unsigned bA = __float_as_uint(h ? tA.y : tA.x), bB = __float_as_uint(h ? tB.y : tB.x);
            if (PAD) {
                bA += bA >> 4;
                bB += bB >> 4;
            }
            const unsigned aA = baseA + 4u * bA, aB = baseB + 4u * bB;
            acc[0][s] += lds_s32(aA) + lds_s32(aB);
            if (NS > 1) acc[1 % NS][s] += lds_s32_off<4 * WIN * (NS > 1 ? 1 : 0)>(aA) + lds_s32_off<4 * WIN * (NS > 1 ? 1 : 0)>(aB);
            if (NS > 2) acc[2 % NS][s] += lds_s32_off<4 * WIN * (NS > 2 ? 2 : 0)>(aA) + lds_s32_off<4 * WIN * (NS > 2 ? 2 : 0)>(aB);
            if (NS > 3) acc[3 % NS][s] += lds_s32_off<4 * WIN * (NS > 3 ? 3 : 0)>(aA) + lds_s32_off<4 * WIN * (NS > 3 ? 3 : 0)>(aB);
        }
    }
}

// Two fast-path views (records g, g2; windows at baseA, baseB) of a ray layout of orientation O.
template <int O, int WIN, int PAD, int NS, int Q>
__device__ __forceinline__ void ws_view_pair(int (&acc)[NS][2 * Q], const float (&lin)[Q], const float (&fix)[2],
                                             float4 g, float4 g2, unsigned baseA, unsigned baseB) {
    constexpr int S = 2 * Q;
    if (O == 0) {   // V: x = lin[q], y = fix[p]
        float2 XA[Q / 2], XB[Q / 2];
#pragma unroll
        for (int k = 0; k < Q / 2; k++) {
            XA[k] = make_float2(fmulr(lin[2 * k], g.x), fmulr(lin[2 * k + 1], g.x));
            XB[k] = make_float2(fmulr(lin[2 * k], g2.x), fmulr(lin[2 * k + 1], g2.x));
        }
        const float2 YA0 = bcast2(faddr(fmulr(fix[0], g.y), g.z)), YA1 = bcast2(faddr(fmulr(fix[1], g.y), g.z));
        const float2 YB0 = bcast2(faddr(fmulr(fix[0], g2.y), g2.z)), YB1 = bcast2(faddr(fmulr(fix[1], g2.y), g2.z));
        ws_gather_two<WIN, PAD, NS, S>(acc, baseA, baseB,
                                       [&](int i) { return add2_rn(XA[i >> 1], (i & 1) ? YA1 : YA0); },
                                       [&](int i) { return add2_rn(XB[i >> 1], (i & 1) ? YB1 : YB0); });
    } else {   // H: x = fix[p], y = lin[q]
        float2 YA[Q / 2], YB[Q / 2];
#pragma unroll
        for (int k = 0; k < Q / 2; k++) {
            YA[k] = make_float2(faddr(fmulr(lin[2 * k], g.y), g.z), faddr(fmulr(lin[2 * k + 1], g.y), g.z));
            YB[k] = make_float2(faddr(fmulr(lin[2 * k], g2.y), g2.z), faddr(fmulr(lin[2 * k + 1], g2.y), g2.z));
        }
        const float2 XA0 = bcast2(fmulr(fix[0], g.x)), XA1 = bcast2(fmulr(fix[1], g.x));
        const float2 XB0 = bcast2(fmulr(fix[0], g2.x)), XB1 = bcast2(fmulr(fix[1], g2.x));
        ws_gather_two<WIN, PAD, NS, S>(acc, baseA, baseB,
                                       [&](int i) { return add2_rn((i & 1) ? XA1 : XA0, YA[i >> 1]); },
                                       [&](int i) { return add2_rn((i & 1) ? XB1 : XB0, YB[i >> 1]); });
    }
}

// one chunk of views: NQ == 0 compact blocks (8 consumer warps; colf/rowf in lin[0..3] /
// lin[4..7]), else the ray layout of orientation O.  Products and y terms are scalar
// (fl(x fcos), fl(fl(y fsin) + foffset)); the per-pixel sums are paired.  Ray layouts take two
// fast-path views at a time where they can; a full chunk whose views are all on the fast path
// (the common case) runs as straight-line code, with one test per chunk.
template <int NQ, int O, int VC, int WIN, int PAD, bool CHECKED, int NS, int NSL, int CW>
__device__ __forceinline__ void ws_consume(int (&acc)[NS][128 / CW], const float (&lin)[64 / CW],
                                           const float (&fix)[2], const int* win, const ViewMeta* meta, int b,
                                           int nv, unsigned& viol) {
    constexpr int Q = 64 / CW, S = 2 * Q;
    if (NQ > 0 && !CHECKED && VC % 2 == 0 && nv == VC) {
        unsigned all = 1u;
#pragma unroll
        for (int vv = 0; vv < VC; vv++) all &= meta[b * VC + vv].off;
        if (all & 1u) {
#pragma unroll 1
            for (int vv = 0; vv < VC; vv += 2) {
                const float4 g = *reinterpret_cast<const float4*>(&meta[b * VC + vv]);
                const float4 g2 = *reinterpret_cast<const float4*>(&meta[b * VC + vv + 1]);
                const unsigned baseA = smem_u32(win + (b * VC + vv) * NSL * WIN) + (__float_as_uint(g.w) & ~3u);
                const unsigned baseB = smem_u32(win + (b * VC + vv + 1) * NSL * WIN) + (__float_as_uint(g2.w) & ~3u);
                ws_view_pair<O, WIN, PAD, NS, Q>(acc, lin, fix, g, g2, baseA, baseB);
            }
            return;
        }
    }
    for (int vv = 0; vv < nv; vv++) {
        const float4 g = *reinterpret_cast<const float4*>(&meta[b * VC + vv]);
        const unsigned offb = __float_as_uint(g.w);
        if (NQ > 0 && !CHECKED && vv + 1 < nv) {
            const float4 g2 = *reinterpret_cast<const float4*>(&meta[b * VC + vv + 1]);
            const unsigned offb2 = __float_as_uint(g2.w);
            if (offb & offb2 & 1u) {
                const unsigned baseA = smem_u32(win + (b * VC + vv) * NSL * WIN) + (offb & ~3u);
                const unsigned baseB = smem_u32(win + (b * VC + vv + 1) * NSL * WIN) + (offb2 & ~3u);
                ws_view_pair<O, WIN, PAD, NS, Q>(acc, lin, fix, g, g2, baseA, baseB);
                vv++;
                continue;
            }
        }
        if (NQ == 0) {   // slot s = 4 r + c: x = lin[c], y = lin[4 + r]
            float2 X[2], Yb[4];
#pragma unroll
            for (int k = 0; k < 2; k++) X[k] = make_float2(fmulr(lin[2 * k], g.x), fmulr(lin[2 * k + 1], g.x));
#pragma unroll
            for (int r = 0; r < 4; r++) Yb[r] = bcast2(faddr(fmulr(lin[(4 + r) % Q], g.y), g.z));
            ws_gather<VC, WIN, PAD, CHECKED, NS, NSL, true, S>(acc, win, meta, b, vv, offb, viol,
                                                               [&](int i) { return add2_rn(X[i & 1], Yb[i >> 1]); });
        } else if (O == 0) {   // V: x = lin[q], y = fix[p]
            float2 X[Q / 2];
#pragma unroll
            for (int k = 0; k < Q / 2; k++) X[k] = make_float2(fmulr(lin[2 * k], g.x), fmulr(lin[2 * k + 1], g.x));
            const float2 Y0 = bcast2(faddr(fmulr(fix[0], g.y), g.z)), Y1 = bcast2(faddr(fmulr(fix[1], g.y), g.z));
            ws_gather<VC, WIN, PAD, CHECKED, NS, NSL, false, S>(
                acc, win, meta, b, vv, offb, viol, [&](int i) { return add2_rn(X[i >> 1], (i & 1) ? Y1 : Y0); });
        } else {   // H: x = fix[p], y = lin[q]
            float2 Y[Q / 2];
#pragma unroll
            for (int k = 0; k < Q / 2; k++)
                Y[k] = make_float2(faddr(fmulr(lin[2 * k], g.y), g.z), faddr(fmulr(lin[2 * k + 1], g.y), g.z));
            const float2 X0 = bcast2(fmulr(fix[0], g.x)), X1 = bcast2(fmulr(fix[1], g.x));
            ws_gather<VC, WIN, PAD, CHECKED, NS, NSL, false, S>(
                acc, win, meta, b, vv, offb, viol, [&](int i) { return add2_rn((i & 1) ? X1 : X0, Y[i >> 1]); });
        }
    }
}

template <int VC, int NB, int PAD, int NS, int CW>
__device__ __forceinline__ void ws_init(int* smi) {
    using Cfg = WsCfg<VC, NB, PAD, NS, CW>;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smi + Cfg::BAR_OFF);
    if (threadIdx.x == 0) {
        for (int b = 0; b < NB; b++) {
            mbar_init(smem_u32(&bars[b]), 1);
            mbar_init(smem_u32(&bars[NB + b]), CW);   // one arrival per consumer warp
        }
        smi[Cfg::ABORT_OFF] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

// One 64x64 tile of NS slices that share the geometry (slice sl: tables J.table + sl * tstride,
// output J.out + sl * ostride) in a buffer layout of NSL windows per view; gc as in
// bp_ref_tile_pipe.
// Returns false (for the whole CTA) after a bounded wait ran out.  Warps 0 .. CW-1 consume, warp
// CW produces.
template <int VC, int NB, int PAD, int NQ, bool CHECKED, int NS = 1, int NSL = NS, int CW = 8>
__device__ __forceinline__ bool bp_ref_tile_ws(const TileJob& J, int* smi, unsigned gc, unsigned* status_counter,
                                               long long tstride = 0, long long ostride = 0) {
    using Cfg = WsCfg<VC, NB, PAD, NSL, CW>;
    constexpr int WIN = Cfg::WIN, Q = Cfg::Q, S = Cfg::S, NC = 32 * CW;
    static_assert(NS <= NSL && NSL <= 4, "the buffer layout holds NSL <= 4 windows per view");
    static_assert(NQ == 0 || Cfg::EXCHANGE_FITS, "the accumulator exchange needs 4096 words per slice in one buffer");
    static_assert(NQ > 0 || CW == 8, "the compact layout is laid out for 8 consumer warps");
    int* win = smi;                                                     // [NB][VC][NSL][WIN]
    ViewMeta* meta = reinterpret_cast<ViewMeta*>(smi + Cfg::META_OFF);  // [NB][VC]
    uint64_t* bars = reinterpret_cast<uint64_t*>(smi + Cfg::BAR_OFF);   // full[NB], empty[NB]
    volatile int* abortw = smi + Cfg::ABORT_OFF;
    const int ixdimp = J.ixdimp;
    const int X0 = J.X0, Y0 = J.Y0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nviews = J.nviews;
    const int nchunks = (nviews + VC - 1) / VC;
    bool failed = false;   // warp-uniform
    int produced = 0;      // producer: chunks of this tile whose fill has been issued
    if (warp == CW) {
        const int nstore = PAD ? ((17 * ixdimp + 3) & ~3) : 16 * ixdimp;
        float4 gg = make_float4(0.0f, 0.0f, 0.0f, 0.0f);   // this chunk's records, lane vv: view vv
        if (nchunks > 0 && lane < min(VC, nviews)) gg = __ldg(J.geom + lane);
        for (; produced < nchunks; produced++) {
            if (__any_sync(0xffffffffu, *abortw != 0)) {
                failed = true;
                break;
            }
            const int v0 = produced * VC, nv = min(VC, nviews - v0);
            const ViewMeta m = view_window<64, 64, WIN, Cfg::ALIGN, PAD>(gg, X0, Y0, nstore);
            if (lane < min(VC, nviews - v0 - VC)) gg = __ldg(J.geom + v0 + VC + lane);
            if (!ws_fill<WIN, VC, NB, NS, NSL>(J, win, meta, bars, v0, nv, gc + (unsigned)produced, lane, m, tstride)) {
                failed = true;
                if (lane == 0) *abortw = 1;
                break;
            }
        }
    } else {
        unsigned viol = 0;
        int acc[NS][S];
#pragma unroll
        for (int sl = 0; sl < NS; sl++)
#pragma unroll
            for (int s = 0; s < S; s++) acc[sl][s] = 0;
        float lin[Q], fix[2];
        int regime = 0;
        float4 gnext = make_float4(0.0f, 0.0f, 0.0f, 0.0f);   // record of the first view of chunk k + 1
        if (NQ > 0) {
            if (nchunks > 0) regime = regime_of<NQ>(__ldg(J.geom));
            if (nchunks > 1) gnext = __ldg(J.geom + VC);
            ray_coords<NQ, CW>(regime, X0, Y0, warp, lane, lin, fix);
        } else {
            const int tx = (warp % 2) * 8 + (lane & 7), ty = (warp / 2) * 4 + (lane >> 3);
#pragma unroll
            for (int c = 0; c < 4; c++) lin[c % Q] = (float)(X0 + tx + 16 * c);
#pragma unroll
            for (int r = 0; r < 4; r++) lin[(4 + r) % Q] = (float)(Y0 + ty + 16 * r);
            fix[0] = fix[1] = 0.0f;
        }
        for (int k = 0; k < nchunks; k++) {
            const unsigned g = gc + (unsigned)k;
            const int b = (int)(g % NB);
            // the producer's abort word is read only when the data wait does not succeed at once
            if (!failed && !__all_sync(0xffffffffu, mbar_try_wait(smem_u32(&bars[b]), (g / NB) & 1u))) {
                if (__any_sync(0xffffffffu, *abortw != 0) ||
                    !__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[b]), (g / NB) & 1u)))
                    failed = true;
            }
            if (!failed) {
                const int nv = min(VC, nviews - k * VC);
                if (NQ == 0 || !(regime & 1))
                    ws_consume<NQ, 0, VC, WIN, PAD, CHECKED, NS, NSL, CW>(acc, lin, fix, win, meta, b, nv, viol);
                else
                    ws_consume<NQ, 1, VC, WIN, PAD, CHECKED, NS, NSL, CW>(acc, lin, fix, win, meta, b, nv, viol);
            } else if (lane == 0) {
                *abortw = 1;
            }
            if (NQ > 0) {
                // the next chunk's regime (the same value in every consumer thread)
                int next = regime;
                if (k + 1 < nchunks) {
                    next = regime_of<NQ>(gnext);
                    if (k + 2 < nchunks) gnext = __ldg(J.geom + (size_t)(k + 2) * VC);
                }
                if (next != regime) {
                    // every consumer is done reading buffer b and none has released it: exchange
                    if (consumers_bar_or<CW>(failed)) {
                        failed = true;
                        break;
                    }
                    // [slices of a round][S slots][NC threads]: all NS slices in one round when the
                    // buffer holds them, else one slice per round
                    int* xs = win + b * VC * NSL * WIN;
                    constexpr int XR = VC * NSL * WIN >= NS * S * NC ? NS : 1;
                    const int on = next & 1, oo = regime & 1;
                    const int shn = ray_shift<NQ>(lane, next);
#pragma unroll
                    for (int r0 = 0; r0 < NS; r0 += XR) {
                        if (r0 > 0) consumers_bar<CW>();   // the previous round's reads are done
#pragma unroll
                        for (int sl = r0; sl < r0 + XR; sl++)
#pragma unroll
                            for (int s = 0; s < S; s++) xs[((sl - r0) * S + s) * NC + tid] = acc[sl][s];
                        consumers_bar<CW>();
#pragma unroll
                        for (int q = 0; q < Q; q++)
#pragma unroll
                            for (int p = 0; p < 2; p++) {
                                const int u = (warp + shn + CW * q) & 63, f = lane + 32 * p;   // new layout
                                const int xr = on ? f : u, yr = on ? u : f;
                                const int a = oo ? xr : yr, c = oo ? yr : xr;                   // old fixed / sheared
                                const int jj = a & 31, pp = a >> 5;
                                const int m = (c - ray_shift<NQ>(jj, regime)) & 63;              // old w + CW q
                                const int src = ((m / CW) * 2 + pp) * NC + (m % CW) * 32 + jj;
#pragma unroll
                                for (int sl = r0; sl < r0 + XR; sl++) acc[sl][2 * q + p] = xs[(sl - r0) * S * NC + src];
                            }
                    }
                    regime = next;
                    ray_coords<NQ, CW>(regime, X0, Y0, warp, lane, lin, fix);
                    // these generic accesses come before the next TMA fill of buffer b
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                }
            }
            if (!failed) {
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&bars[NB + b]));
            }
        }
        // Output: the accumulators go through shared memory into row order, then every row of
        // the tile leaves as coalesced 16-byte stores (8-byte-aligned-free fallback: 4-byte
        // stores, still row order).  All consumers are past their last chunk (the barrier), the
        // producer has issued its last fill, so the window buffers are free.
        if (!consumers_bar_or<CW>(failed)) {
            if (CHECKED && viol) atomicAdd(status_counter, viol);
            constexpr int RS = 68;                                  // row stride in words (16-byte rows)
            int* stg = win;                                         // [NS][64][RS]
            static_assert(NS * 64 * RS <= NB * VC * NSL * WIN, "the output staging fits the buffers");
            const int sh = NQ > 0 ? ray_shift<NQ>(lane, regime) : 0;
            const int tx = (warp % 2) * 8 + (lane & 7), ty = (warp / 2) * 4 + (lane >> 3);
#pragma unroll
            for (int s = 0; s < S; s++) {
                int x, y;
                if (NQ == 0) {
                    x = tx + 16 * (s & 3);
                    y = ty + 16 * (s >> 2);
                } else {
                    const int u = (warp + sh + CW * (s >> 1)) & 63, f = lane + 32 * (s & 1);
                    x = (regime & 1) ? f : u;
                    y = (regime & 1) ? u : f;
                }
#pragma unroll
                for (int sl = 0; sl < NS; sl++) stg[(sl * 64 + y) * RS + x] = acc[sl][s];
            }
            consumers_bar<CW>();
            const bool vec = !J.accumulate && (ixdimp & 3) == 0 && !(reinterpret_cast<uintptr_t>(J.out) & 15) &&
                             !(ostride & 3);
            for (int e = tid; e < NS * 64 * 16; e += NC) {   // 16 four-pixel groups per row
                const int sl = e >> 10, y = (e >> 4) & 63, x = (e & 15) * 4;
                const int gy = Y0 + y, gx = X0 + x;
                if (gy >= ixdimp || gx >= ixdimp) continue;
                const int4 v = *reinterpret_cast<const int4*>(stg + (sl * 64 + y) * RS + x);
                int* o = J.out + sl * ostride + (size_t)gy * ixdimp + gx;
                if (vec) {
                    *reinterpret_cast<int4*>(o) = v;
                } else {
                    const int w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        if (gx + i < ixdimp) {
                            if (J.accumulate) atomicAdd(o + i, w4[i]);   // int sums: any order gives the same slice
                            else o[i] = w4[i];
                        }
                }
            }
        } else {
            failed = true;
        }
    }
    if (__syncthreads_or(failed)) {
        if (tid == 0) atomicOr(&g_kernel_status, 1u);
        // the producer's fills up to chunk `produced`: give them a bounded chance to land before
        // the CTA can leave
        if (warp == CW) {
            for (int c = produced > NB ? produced - NB : 0; c < produced; c++) {
                const unsigned g = gc + (unsigned)c;
                mbar_wait_bounded(smem_u32(&bars[g % NB]), (g / NB) & 1u);
            }
        }
        return false;
    }
    return true;
}

// grid (tiles, slices / NS): CTA row y covers slices slice0 + NS y (.. + NS - 1); NS > 1 needs
// slices that share the geometry (geom_slice_stride 0)
template <int VC, int NB, int PAD, int NQ, int MINB, bool CHECKED, int NS = 1, int CW = 8>
__global__ void __launch_bounds__(32 * CW + 32, MINB) k_bp_ref_ws(BackprojLaunch p, int slice0) {
    extern __shared__ __align__(128) int smi[];
    ws_init<VC, NB, PAD, NS, CW>(smi);
    __syncthreads();
    const int tiles_x = (p.ixdimp + 63) / 64;
    const int sl = slice0 + NS * (int)blockIdx.y;
    TileJob J;
    J.table = p.table + (size_t)sl * p.slice_table_stride;
    J.geom = p.geom + (size_t)sl * p.geom_slice_stride;
    J.out = static_cast<int*>(p.out) + (size_t)sl * p.out_slice_stride;
    J.table_stride = p.table_stride;
    J.nviews = p.nviews;
    J.ixdimp = p.ixdimp;
    J.X0 = (blockIdx.x % tiles_x) * 64;
    J.Y0 = (blockIdx.x / tiles_x) * 64;
    J.pair = NS > 1;
    J.accumulate = 0;
    if (gridDim.z > 1) {   // view group blockIdx.z of gridDim.z: partial sums added into the slice
        const int v0 = (int)(((long long)p.nviews * blockIdx.z) / gridDim.z);
        const int v1 = (int)(((long long)p.nviews * (blockIdx.z + 1)) / gridDim.z);
        J.table += (size_t)v0 * p.table_stride;
        J.geom += v0;
        J.nviews = v1 - v0;
        J.accumulate = 1;
    }
    bp_ref_tile_ws<VC, NB, PAD, NQ, CHECKED, NS, NS, CW>(J, smi, 0u, p.status_counter, p.slice_table_stride,
                                                         p.out_slice_stride);
}

// NSL = 2: jobs may cover slice pairs (TileJob::pair), in a layout with two windows per view
template <int VC, int NB, int PAD, int NQ, int MINB, int NSL = 1, int CW = 8>
__global__ void __launch_bounds__(32 * CW + 32, MINB) k_bp_ref_ws_persistent(const TileJob* jobs, int njobs,
                                                                             unsigned* counter) {
    extern __shared__ __align__(128) int smi[];
    __shared__ int s_item;
    ws_init<VC, NB, PAD, NSL, CW>(smi);
    unsigned gc = 0;
    for (;;) {
        if (threadIdx.x == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= njobs) break;
        const TileJob J = jobs[it];
        bool ok;
        if (NSL > 2 && J.pair >= 2)
            ok = bp_ref_tile_ws<VC, NB, PAD, NQ, false, (NSL > 2 ? 3 : 1), NSL, CW>(
                J, smi, gc, nullptr, (long long)J.nviews * J.table_stride, (long long)J.ixdimp * J.ixdimp);
        else if (NSL > 1 && J.pair)
            ok = bp_ref_tile_ws<VC, NB, PAD, NQ, false, (NSL > 1 ? 2 : 1), NSL, CW>(
                J, smi, gc, nullptr, (long long)J.nviews * J.table_stride, (long long)J.ixdimp * J.ixdimp);
        else
            ok = bp_ref_tile_ws<VC, NB, PAD, NQ, false, 1, NSL, CW>(J, smi, gc, nullptr);
        if (!ok) return;   // CTA-uniform
        gc += (unsigned)((J.nviews + VC - 1) / VC);
    }
}

// ---- LIN / FP16 / BF16: linear interpolation of filtered pair rows -------------------------------
// Not the reference's arithmetic (that is REF): the filtered row of each view is stored as pairs
// (r[j], r[j+1] - r[j]) in FP32 (8 B) or, with a per-row scale, FP16 / BF16 (4 B), and every update
// interpolates at the FP32 detector coordinate u:  acc += scale * (r[j] + (u - j) * slope[j]).
// Same warp-decoupled pipeline as bp_ref_tile_pipe: each view's window of pairs (the detector
// pixels a tile can touch) is staged by one TMA bulk copy into NB buffers with full/empty
// mbarriers, so 16-bit storage halves both the L2 traffic and the shared-memory gathers.
// Per update: FADD (u), FADD.RZ (floor as bits), FADD (j as float), FADD (fraction), LEA, LDS,
// [2 conversions], FFMA, FFMA.
template <int MODE>
struct LinElem;
template <>
struct LinElem<RV_MODE_LIN> { static constexpr int ES = 8; };
template <>
struct LinElem<RV_MODE_LIN_F16> { static constexpr int ES = 4; };
template <>
struct LinElem<RV_MODE_LIN_BF16> { static constexpr int ES = 4; };

// the pair at byte address addr + OFF (OFF in the instruction)
template <int MODE, int OFF = 0>
__device__ __forceinline__ float2 lin_pair(unsigned addr) {
    if (MODE == RV_MODE_LIN) {
        float2 v;
        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];" : "=f"(v.x), "=f"(v.y) : "r"(addr), "n"(OFF));
        return v;
    } else {
        unsigned w;
        asm volatile("ld.shared.u32 %0, [%1+%2];" : "=r"(w) : "r"(addr), "n"(OFF));
        if (MODE == RV_MODE_LIN_F16) {
            __half2 h = *reinterpret_cast<__half2*>(&w);
            return __half22float2(h);
        }
        return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
    }
}

// 16-bit rows: acc += r + f * slope as a mixed-precision FMA and add (16-bit operands, FP32
// arithmetic and result, one rounding each), with the fraction f rounded to the row format once
// per pixel -- three instructions per slice-update with the gather, as the FP32 form.  BF16 rows
// are stored unscaled; FP16 rows carry one power-of-two scale per filter, applied exactly to the
// finished sums (lin_store).
template <int MODE>
__device__ __forceinline__ unsigned short half_bits(float f) {
    unsigned short h;
    if (MODE == RV_MODE_LIN_BF16) asm("cvt.rn.bf16.f32 %0, %1;" : "=h"(h) : "f"(f));
    else asm("cvt.rn.f16.f32 %0, %1;" : "=h"(h) : "f"(f));
    return h;
}
template <int MODE, int OFF>
__device__ __forceinline__ void lin_add_half(float& acc, unsigned addr, unsigned short fb) {
    unsigned w;
    asm volatile("ld.shared.u32 %0, [%1+%2];" : "=r"(w) : "r"(addr), "n"(OFF));
    if (MODE == RV_MODE_LIN_BF16)
        asm("{\n .reg .b16 r, d;\n .reg .f32 t;\n mov.b32 {r, d}, %1;\n fma.rn.f32.bf16 t, d, %2, %3;\n"
            " add.rn.f32.bf16 %0, r, t;\n}\n"
            : "=f"(acc)
            : "r"(w), "h"(fb), "f"(acc));
    else
        asm("{\n .reg .b16 r, d;\n .reg .f32 t;\n mov.b32 {r, d}, %1;\n fma.rn.f32.f16 t, d, %2, %3;\n"
            " add.rn.f32.f16 %0, r, t;\n}\n"
            : "=f"(acc)
            : "r"(w), "h"(fb), "f"(acc));
}

// NS windows per view (slices that share the geometry, one after the other), NS scales per view
template <int WX, int WY, int RX, int RY, int VC, int NB, int MODE, int NS = 1>
struct LinCfg {
    static constexpr int VC_ = VC, NB_ = NB, RX_ = RX, RY_ = RY, NS_ = NS;
    static constexpr int NT = 32 * WX * WY, NW = NT / 32;
    static constexpr int GX = 8 * WX, GY = 4 * WY, TX = GX * RX, TY = GY * RY;
    static constexpr int ES = LinElem<MODE>::ES;
    // detector-pixel span of a tile + margins (2 below, 3 above) + 4-pair alignment, in pairs
    static constexpr int WINP = ((isqrt_ceil((TX - 1) * (TX - 1) + (TY - 1) * (TY - 1)) + 2 + 3 + 4 + 4) + 15) / 16 * 16;
    static constexpr int WIN_BYTES = WINP * ES;
    static constexpr int META_OFF = NB * VC * NS * WIN_BYTES;             // bytes
    static constexpr int BAR_OFF = META_OFF + NB * VC * (int)sizeof(ViewMeta);
    static constexpr size_t SMEM = (size_t)BAR_OFF + (size_t)2 * NB * 8;
    static constexpr int SCL_OFF = BAR_OFF + 2 * NB * 8;                  // float scales [NB][VC][NS]
    static constexpr int ABORT_OFF = SCL_OFF + NB * VC * NS * 4;
    static constexpr size_t SMEM_WS = (size_t)ABORT_OFF + 16;   // the producer-warp form
};

// Per-CTA state of a LIN tile: the slice's pair rows, scales and FP64 geometry, and the tile.
struct LinTile {
    const unsigned char* rows;
    const float* scales;
    const LinGeom* geom;
    int X0, Y0, nviews, ixdimp;
    long long row_stride;
    long long slice_row_bytes;    // bytes between the rows of consecutive slices
};
__device__ __forceinline__ LinTile lin_tile(const BackprojLaunch& p, int TX, int TY, int ES, int slice) {
    LinTile t;
    const int tiles_x = (p.ixdimp + TX - 1) / TX;
    t.X0 = (blockIdx.x % tiles_x) * TX;
    t.Y0 = (blockIdx.x / tiles_x) * TY;
    t.rows = static_cast<const unsigned char*>(p.rows16) + (size_t)slice * p.slice_row_stride * ES;
    t.scales = p.row_scale ? p.row_scale + (size_t)slice * p.nviews : nullptr;
    t.geom = p.geom64 + (size_t)slice * p.geom_slice_stride;
    t.slice_row_bytes = p.slice_row_stride * ES;
    t.nviews = p.nviews;
    t.ixdimp = p.ixdimp;
    t.row_stride = p.row_stride;
    return t;
}

// The LIN record of view v: its FP64 geometry and the scales of its NS slices (slice sl's scales
// follow at sl * nviews).
template <typename Cfg>
__device__ __forceinline__ void lin_load(const LinTile& T, int v, LinGeom& gg, float (&sc)[Cfg::NS_]) {
    gg = T.geom[v];
#pragma unroll
    for (int sl = 0; sl < Cfg::NS_; sl++) sc[sl] = T.scales ? T.scales[(size_t)sl * T.nviews + v] : 1.0f;
}
// The window record of a view for the tile: u at the tile origin in FP64 (two FMAs); the tile's
// lowest u adds the negative parts of the tile's extent, which FP32 gives well inside the
// window's 2-pixel margin.  sc0: slice 0's scale (kept in the record's fourth word).
template <typename Cfg>
__device__ __forceinline__ ViewMeta lin_record(const LinTile& T, const LinGeom& gg, float sc0) {
    constexpr int TX = Cfg::TX, TY = Cfg::TY, WINP = Cfg::WINP;
    const double base = fma((double)T.X0, gg.c, fma((double)T.Y0, gg.s, gg.off));
    const float lo = (float)base + fminf(0.0f, (float)(TX - 1) * (float)gg.c) + fminf(0.0f, (float)(TY - 1) * (float)gg.s);
    const int ilo = (int)floorf(lo) - 2;
    const int w0 = ilo >= 0 ? (ilo & ~3) : -((-ilo + 3) & ~3);
    ViewMeta m;
    m.w0 = w0;
    m.nwin = WINP;
    m.a = max(w0, 0);
    m.b = min(w0 + WINP, (T.ixdimp + 3) & ~3);
    m.gc = (float)gg.c;
    m.gs = (float)gg.s;
    m.go = (float)(base - (double)w0);   // window-relative u at the tile origin
    m.off = __float_as_uint(sc0);
    return m;
}

// Publish chunk c's records (lane vv: view vv's record m and slice scales sc) in buffer c % NB
// once its empty barrier shows every consumer is done with it, zero-fill the window parts outside
// the rows (edge tiles only), and issue the bulk copies -- lane vv those of view vv -- on the
// buffer's full barrier.  False (warp-uniform) when the bounded wait ran out.
template <typename Cfg>
__device__ __forceinline__ bool lin_publish(const LinTile& T, unsigned char* smb, ViewMeta* meta, uint64_t* bars,
                                            int c, int lane, int nv, const ViewMeta& m,
                                            const float (&sc)[Cfg::NS_], float* scl) {
    constexpr int NB = Cfg::NB_, VC = Cfg::VC_, ES = Cfg::ES, NS = Cfg::NS_;
    const unsigned g = (unsigned)c;
    const int b = (int)(g % NB);
    if (!__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[NB + b]), ((g / NB) & 1u) ^ 1u)))
        return false;
    const int v0 = c * VC;
    const bool mine = lane < nv;
    if (mine) {
        meta[b * VC + lane] = m;
        if (NS > 1 && scl) {
#pragma unroll
            for (int sl = 0; sl < NS; sl++) scl[(b * VC + lane) * NS + sl] = sc[sl];
        }
    }
    unsigned edges = __ballot_sync(0xffffffffu, mine && !(m.a == m.w0 && m.b == m.w0 + m.nwin));
    while (edges) {   // warp-uniform
        const int vv = __ffs(edges) - 1;
        edges &= edges - 1;
        const int w0 = __shfl_sync(0xffffffffu, m.w0, vv), nwin = __shfl_sync(0xffffffffu, m.nwin, vv);
        const int a = __shfl_sync(0xffffffffu, m.a, vv), e1 = __shfl_sync(0xffffffffu, m.b, vv);
        const int bytes_a = (e1 > a ? a - w0 : nwin) * ES, bytes_b = (e1 > a ? e1 - w0 : nwin) * ES;
#pragma unroll
        for (int sl = 0; sl < NS; sl++) {
            int4* w4 = reinterpret_cast<int4*>(smb + (size_t)((b * VC + vv) * NS + sl) * Cfg::WIN_BYTES);
            for (int e = lane; e < bytes_a / 16; e += 32) w4[e] = make_int4(0, 0, 0, 0);
            for (int e = bytes_b / 16 + lane; e < Cfg::WIN_BYTES / 16; e += 32) w4[e] = make_int4(0, 0, 0, 0);
        }
    }
    const bool copy = mine && m.b > m.a;
    const unsigned bytes = __reduce_add_sync(0xffffffffu, copy ? (unsigned)(NS * (m.b - m.a) * ES) : 0u);
    // the records and zero fills are ordered before the barrier's completion, and every lane's
    // generic accesses to the buffer before its own copies into it
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncwarp();
    const unsigned bar = smem_u32(&bars[b]);
    if (lane == 0) mbar_arrive_expect_tx(bar, bytes);
    __syncwarp();
    if (copy) {
#pragma unroll
        for (int sl = 0; sl < NS; sl++) {
            const unsigned char* src = T.rows + sl * T.slice_row_bytes + ((size_t)(v0 + lane) * T.row_stride + m.a) * ES;
            const unsigned dst = smem_u32(smb + (size_t)((b * VC + lane) * NS + sl) * Cfg::WIN_BYTES + (m.a - m.w0) * ES);
            tma_bulk_g2s(dst, src, (unsigned)((m.b - m.a) * ES), bar);
        }
    }
    return true;
}

// One warp fills buffer c % NB with the pair windows of chunk c (views c*VC ..): records, then
// lin_publish.  False (warp-uniform) when the bounded wait ran out.
template <typename Cfg>
__device__ __forceinline__ bool lin_fill(const LinTile& T, unsigned char* smb, ViewMeta* meta, uint64_t* bars, int c,
                                         int lane, float* scl = nullptr) {
    const int v0 = c * Cfg::VC_;
    const int nv = min(Cfg::VC_, T.nviews - v0);
    LinGeom gg{};
    float sc[Cfg::NS_];
#pragma unroll
    for (int sl = 0; sl < Cfg::NS_; sl++) sc[sl] = 1.0f;
    if (lane < nv) lin_load<Cfg>(T, v0 + lane, gg, sc);
    const ViewMeta m = lin_record<Cfg>(T, gg, sc[0]);
    return lin_publish<Cfg>(T, smb, meta, bars, c, lane, nv, m, sc, scl);
}

// one slice's update of a pixel: acc += (scaled) r + f * slope, from the pair at addr + sl windows
template <typename Cfg, int MODE, int SL>
__device__ __forceinline__ void lin_slice(float& acc, unsigned addr, float f, float sc, unsigned short fb) {
    if (MODE != RV_MODE_LIN) {
        lin_add_half<MODE, SL * Cfg::WIN_BYTES>(acc, addr, fb);
        return;
    }
    const float2 q = lin_pair<MODE, SL * Cfg::WIN_BYTES>(addr);
    const float v = fmaf(f, q.y, q.x);
    if (MODE == RV_MODE_LIN) acc += v;
    else acc = fmaf(v, sc, acc);
}

// acc[sl] += the interpolated, scaled row value of every pixel of the thread in slice sl, for the
// nv views of buffer b.  The NS slices share the geometry, so each pixel's detector coordinate,
// window index and fraction are computed once (scl: the per-slice scales when NS > 1).
template <typename Cfg, int MODE>
__device__ __forceinline__ void lin_consume(float (&acc)[Cfg::NS_][Cfg::RY_][Cfg::RX_], const float (&colf)[Cfg::RX_],
                                            const float (&rowf)[Cfg::RY_], const unsigned char* smb,
                                            const ViewMeta* meta, int b, int nv, const float* scl = nullptr) {
    constexpr int RX = Cfg::RX_, RY = Cfg::RY_, VC = Cfg::VC_, ES = Cfg::ES, NS = Cfg::NS_;
    for (int vv = 0; vv < nv; vv++) {
        const float4 gm = *reinterpret_cast<const float4*>(&meta[b * VC + vv]);
        float sc[NS];
        sc[0] = __uint_as_float(__float_as_uint(gm.w));
#pragma unroll
        for (int sl = 1; sl < NS; sl++) sc[sl] = scl[(b * VC + vv) * NS + sl];
        static_assert(RX % 2 == 0, "pixel columns go in pairs");
        float2 xv[RX / 2];
        float yv[RY];
#pragma unroll
        for (int c = 0; c < RX / 2; c++) xv[c] = make_float2(fmulr(colf[2 * c], gm.x), fmulr(colf[2 * c + 1], gm.x));
#pragma unroll
        for (int r = 0; r < RY; r++) yv[r] = fmaf(rowf[r], gm.y, gm.z);
        // address of pair 0 minus the 2^23 bit pattern (unsigned wrap-around)
        const unsigned base = smem_u32(smb + (size_t)(b * VC + vv) * NS * Cfg::WIN_BYTES) - (unsigned)ES * kMagicBits;
        const float2 mag = make_float2(8388608.0f, 8388608.0f);
#pragma unroll
        for (int r = 0; r < RY; r++)
#pragma unroll
            for (int c2 = 0; c2 < RX / 2; c2++) {
                // two pixels per instruction: u, its floor as bits (the 2^23 add), the fraction
                const float2 u2 = add2_rn(xv[c2], bcast2(yv[r]));        // >= 1.9 inside the window
                const float2 t2 = add2_rz(u2, mag);
                const float2 f2 = sub2_rn(u2, sub2_rn(t2, mag));
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int c = 2 * c2 + h;
                const unsigned bits = __float_as_uint(h ? t2.y : t2.x);
                const float f = h ? f2.y : f2.x;
                const unsigned a = base + (unsigned)ES * bits;
                const unsigned short fb = MODE != RV_MODE_LIN ? half_bits<MODE>(f) : (unsigned short)0;
                lin_slice<Cfg, MODE, 0>(acc[0][r][c], a, f, sc[0], fb);
                if (NS > 1) lin_slice<Cfg, MODE, (NS > 1 ? 1 : 0)>(acc[1 % NS][r][c], a, f, sc[1 % NS], fb);
                if (NS > 2) lin_slice<Cfg, MODE, (NS > 2 ? 2 : 0)>(acc[2 % NS][r][c], a, f, sc[2 % NS], fb);
                if (NS > 3) lin_slice<Cfg, MODE, (NS > 3 ? 3 : 0)>(acc[3 % NS][r][c], a, f, sc[3 % NS], fb);
            }
            }
    }
}

template <typename Cfg>
__device__ __forceinline__ void lin_store(const BackprojLaunch& p, const LinTile& T, int slice,
                                          const float (&acc)[Cfg::NS_][Cfg::RY_][Cfg::RX_], int tx, int ty) {
#pragma unroll
    for (int sl = 0; sl < Cfg::NS_; sl++) {
        float* out = static_cast<float*>(p.out) + (size_t)(slice + sl) * p.out_slice_stride;
        // FP16 sums are in units of the slice's power-of-two row scale (every row of a slice has
        // the same one): scaling them is exact
        const float sc = (p.mode == RV_MODE_LIN_F16 && T.scales) ? T.scales[(size_t)sl * T.nviews] : 1.0f;
#pragma unroll
        for (int r = 0; r < Cfg::RY_; r++) {
            const int y = T.Y0 + ty + Cfg::GY * r;
            if (y >= T.ixdimp) continue;
#pragma unroll
            for (int c = 0; c < Cfg::RX_; c++) {
                const int x = T.X0 + tx + Cfg::GX * c;
                if (x < T.ixdimp) out[(size_t)y * T.ixdimp + x] = acc[sl][r][c] * sc;
            }
        }
    }
}

// Warp 0 produces as well as consumes (the layout of the REF pipeline's variant 11).
template <int WX, int WY, int RX, int RY, int VC, int NB, int MODE, int MINB>
__global__ void __launch_bounds__(32 * WX * WY, MINB) k_bp_lin_pipe(BackprojLaunch p) {
    using Cfg = LinCfg<WX, WY, RX, RY, VC, NB, MODE>;
    extern __shared__ __align__(128) unsigned char smb[];
    ViewMeta* meta = reinterpret_cast<ViewMeta*>(smb + Cfg::META_OFF);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smb + Cfg::BAR_OFF);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int b = 0; b < NB; b++) {
            mbar_init(smem_u32(&bars[b]), 1);
            mbar_init(smem_u32(&bars[NB + b]), Cfg::NW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const LinTile T = lin_tile(p, Cfg::TX, Cfg::TY, Cfg::ES, blockIdx.y);
    const int tx = (warp % WX) * 8 + (lane & 7), ty = (warp / WX) * 4 + (lane >> 3);
    const int nchunks = (T.nviews + VC - 1) / VC;
    // coordinates relative to the tile origin (small, so FP32 keeps ~1e-6 px); the tile-origin term
    // of each view comes from the FP64 geometry
    float colf[RX], rowf[RY];
#pragma unroll
    for (int c = 0; c < RX; c++) colf[c] = (float)(tx + Cfg::GX * c);
#pragma unroll
    for (int r = 0; r < RY; r++) rowf[r] = (float)(ty + Cfg::GY * r);
    float acc[1][RY][RX];
#pragma unroll
    for (int r = 0; r < RY; r++)
#pragma unroll
        for (int c = 0; c < RX; c++) acc[0][r][c] = 0.0f;
    bool ok = true;
    int produced = 0;
    if (warp == 0)
        for (; produced < nchunks && produced < NB - 1; produced++)
            if (!lin_fill<Cfg>(T, smb, meta, bars, produced, lane)) { ok = false; break; }
    for (int k = 0; ok && k < nchunks; k++) {
        if (warp == 0 && produced < nchunks) {
            if (!lin_fill<Cfg>(T, smb, meta, bars, produced, lane)) { ok = false; break; }
            produced++;
        }
        const unsigned g = (unsigned)k;
        const int b = (int)(g % NB);
        if (!__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[b]), (g / NB) & 1u))) { ok = false; break; }
        lin_consume<Cfg, MODE>(acc, colf, rowf, smb, meta, b, min(VC, T.nviews - k * VC));
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&bars[NB + b]));
    }
    if (!ok) {
        atomicOr(&g_kernel_status, 1u);
        if (warp == 0)
            for (int c = produced > NB ? produced - NB : 0; c < produced; c++)
                mbar_wait_bounded(smem_u32(&bars[(unsigned)c % NB]), ((unsigned)c / NB) & 1u);
        return;
    }
    lin_store<Cfg>(p, T, blockIdx.y, acc, tx, ty);
}

// A ninth warp only produces (as the REF kernel's variant 16); the eight consumer warps do the
// same work and never wait for a fill a busy consumer has not issued.  NS > 1: the CTA takes NS
// slices that share the geometry (slice0 + NS * blockIdx.y ..) and shares each pixel's index
// arithmetic between them.  A consumer whose bounded wait ran out raises the abort word and
// leaves its loop (the consumers share no barrier here); all 288 threads meet at one block
// barrier at the end.
template <int VC, int NB, int MODE, int MINB, int NS = 1>
__global__ void __launch_bounds__(288, MINB) k_bp_lin_ws(BackprojLaunch p, int slice0) {
    using Cfg = LinCfg<2, 4, 4, 4, VC, NB, MODE, NS>;
    static_assert(Cfg::NT == 256, "8 consumer warps");
    extern __shared__ __align__(128) unsigned char smb[];
    ViewMeta* meta = reinterpret_cast<ViewMeta*>(smb + Cfg::META_OFF);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smb + Cfg::BAR_OFF);
    float* scl = reinterpret_cast<float*>(smb + Cfg::SCL_OFF);
    volatile int* abortw = reinterpret_cast<volatile int*>(smb + Cfg::ABORT_OFF);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int b = 0; b < NB; b++) {
            mbar_init(smem_u32(&bars[b]), 1);
            mbar_init(smem_u32(&bars[NB + b]), 8);
        }
        *abortw = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const int slice = slice0 + NS * (int)blockIdx.y;
    const LinTile T = lin_tile(p, Cfg::TX, Cfg::TY, Cfg::ES, slice);
    const int nchunks = (T.nviews + VC - 1) / VC;
    bool failed = false;
    int produced = 0;
    if (warp == 8) {
        // the records of chunk produced + 1 are loaded while chunk produced waits for its buffer
        LinGeom gg{};
        float sc[NS];
#pragma unroll
        for (int sl = 0; sl < NS; sl++) sc[sl] = 1.0f;
        if (nchunks > 0 && lane < min(VC, T.nviews)) lin_load<Cfg>(T, lane, gg, sc);
        for (; produced < nchunks; produced++) {
            if (__any_sync(0xffffffffu, *abortw != 0)) { failed = true; break; }
            const int v0 = produced * VC, nv = min(VC, T.nviews - v0);
            const ViewMeta m = lin_record<Cfg>(T, gg, sc[0]);
            float cur[NS];
#pragma unroll
            for (int sl = 0; sl < NS; sl++) cur[sl] = sc[sl];
            if (lane < min(VC, T.nviews - v0 - VC)) lin_load<Cfg>(T, v0 + VC + lane, gg, sc);
            if (!lin_publish<Cfg>(T, smb, meta, bars, produced, lane, nv, m, cur, scl)) {
                failed = true;
                if (lane == 0) *abortw = 1;
                break;
            }
        }
    } else {
        const int tx = (warp % 2) * 8 + (lane & 7), ty = (warp / 2) * 4 + (lane >> 3);
        float colf[4], rowf[4];
#pragma unroll
        for (int c = 0; c < 4; c++) colf[c] = (float)(tx + Cfg::GX * c);
#pragma unroll
        for (int r = 0; r < 4; r++) rowf[r] = (float)(ty + Cfg::GY * r);
        float acc[NS][4][4];
#pragma unroll
        for (int sl = 0; sl < NS; sl++)
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int c = 0; c < 4; c++) acc[sl][r][c] = 0.0f;
        for (int k = 0; k < nchunks; k++) {
            const unsigned g = (unsigned)k;
            const int b = (int)(g % NB);
            if (__any_sync(0xffffffffu, *abortw != 0) ||
                !__all_sync(0xffffffffu, mbar_wait_bounded(smem_u32(&bars[b]), (g / NB) & 1u))) {
                failed = true;
                if (lane == 0) *abortw = 1;
                break;
            }
            lin_consume<Cfg, MODE>(acc, colf, rowf, smb, meta, b, min(VC, T.nviews - k * VC), scl);
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&bars[NB + b]));
        }
        if (!failed) lin_store<Cfg>(p, T, slice, acc, tx, ty);
    }
    if (__syncthreads_or(failed)) {
        if (tid == 0) atomicOr(&g_kernel_status, 1u);
        if (warp == 8)
            for (int c = produced > NB ? produced - NB : 0; c < produced; c++)
                mbar_wait_bounded(smem_u32(&bars[(unsigned)c % NB]), ((unsigned)c / NB) & 1u);
    }
}

template <int MODE>
static cudaError_t go_lin(const BackprojLaunch& p, cudaStream_t s) {
    constexpr int WX = 2, WY = 4, RX = 4, RY = 4, VC = 8, NB = 2, MINB = 4;
    using Cfg = LinCfg<WX, WY, RX, RY, VC, NB, MODE>;
    auto kern = k_bp_lin_pipe<WX, WY, RX, RY, VC, NB, MODE, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM);
    if (e != cudaSuccess) return e;
    const int tiles = ((p.ixdimp + Cfg::TX - 1) / Cfg::TX) * ((p.ixdimp + Cfg::TY - 1) / Cfg::TY);
    kern<<<dim3(tiles, p.nslices), Cfg::NT, Cfg::SMEM, s>>>(p);
    t_bp_launches++;
    return cudaGetLastError();
}

template <int MODE, int VC, int NB, int MINB, int NS = 1>
static cudaError_t go_lin_ws_rows(const BackprojLaunch& p, cudaStream_t s, int slice0, int rows) {
    using Cfg = LinCfg<2, 4, 4, 4, VC, NB, MODE, NS>;
    auto kern = k_bp_lin_ws<VC, NB, MODE, MINB, NS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM_WS);
    if (e != cudaSuccess) return e;
    const int tiles = ((p.ixdimp + Cfg::TX - 1) / Cfg::TX) * ((p.ixdimp + Cfg::TY - 1) / Cfg::TY);
    kern<<<dim3(tiles, rows), 288, Cfg::SMEM_WS, s>>>(p, slice0);
    t_bp_launches++;
    return cudaGetLastError();
}

template <int MODE, int VC, int NB, int MINB>
static cudaError_t go_lin_ws(const BackprojLaunch& p, cudaStream_t s) {
    return go_lin_ws_rows<MODE, VC, NB, MINB>(p, s, 0, p.nslices);
}

// slice pairs when the slices share the geometry (an odd last slice, or per-slice geometry, runs
// one slice per CTA)
template <int MODE>
static cudaError_t go_lin_ws_pairs(const BackprojLaunch& p, cudaStream_t s) {
    if (p.geom_slice_stride != 0 || p.nslices < 2) return go_lin_ws<MODE, 8, 2, 4>(p, s);
    cudaError_t e = go_lin_ws_rows<MODE, 8, 2, 2, 2>(p, s, 0, p.nslices / 2);
    if (e == cudaSuccess && (p.nslices & 1)) e = go_lin_ws_rows<MODE, 8, 2, 4>(p, s, p.nslices - 1, 1);
    return e;
}

// groups of three slices per CTA, the rest as pairs (n = 3t, 3t + 2 or 3(t - 1) + 4); fewer than
// three slices, or per-slice geometry, go to the pair form
template <int MODE>
static cudaError_t go_lin_ws_triples(const BackprojLaunch& p, cudaStream_t s) {
    if (p.geom_slice_stride != 0 || p.nslices < 3) return go_lin_ws_pairs<MODE>(p, s);
    int t3 = p.nslices / 3;
    if (p.nslices % 3 == 1) t3--;
    cudaError_t e = t3 > 0 ? go_lin_ws_rows<MODE, 8, 2, 2, 3>(p, s, 0, t3) : cudaSuccess;
    const int rest = p.nslices - 3 * t3;
    if (e == cudaSuccess && rest >= 2) e = go_lin_ws_rows<MODE, 8, 2, 2, 2>(p, s, 3 * t3, rest / 2);
    if (e == cudaSuccess && (rest & 1)) e = go_lin_ws_rows<MODE, 8, 2, 4>(p, s, p.nslices - 1, 1);
    return e;
}

// LIN kernel form (RV_LIN_VARIANT): 0 = warp 0 also produces, 2 buffers x 8 views; 1 = a
// dedicated producer warp, 2 x 8; 2 = producer warp, 3 x 8, 3 CTAs/SM; 3 = producer warp, 2 x 16;
// 4 = producer warp and slice pairs; 5 = producer warp and slice triples.  Default: pairs for
// FP32 rows (three 8-byte gathers per index measured slower: 116 against 110 ms per 64-slice
// step), triples for the 16-bit rows (FP16 141 -> 130 ms, BF16 121 -> 98 ms).
template <int MODE>
static cudaError_t dispatch_lin(const BackprojLaunch& p, cudaStream_t s) {
    static const int env = env_int("RV_LIN_VARIANT", -1);
    const int v = env >= 0 ? env : (MODE == RV_MODE_LIN ? 4 : 5);
    switch (v) {
    case 0: return go_lin<MODE>(p, s);
    case 2: return go_lin_ws<MODE, 8, 3, 3>(p, s);
    case 3: return go_lin_ws<MODE, 16, 2, 3>(p, s);
    case 4: return go_lin_ws_pairs<MODE>(p, s);
    case 5: return go_lin_ws_triples<MODE>(p, s);
    default: return go_lin_ws<MODE, 8, 2, 4>(p, s);
    }
}

cudaError_t launch_bp_lin(const BackprojLaunch& p, cudaStream_t s) {
    switch (p.mode) {
    case RV_MODE_LIN: return dispatch_lin<RV_MODE_LIN>(p, s);
    case RV_MODE_LIN_F16: return dispatch_lin<RV_MODE_LIN_F16>(p, s);
    case RV_MODE_LIN_BF16: return dispatch_lin<RV_MODE_LIN_BF16>(p, s);
    default: return cudaErrorInvalidValue;
    }
}

// ---- pair-table variant ------------------------------------------------------------------------
// The table holds, per detector pixel j, the float pair (p0, p1p0) from which the reference builds
// its 16 ints (source/general.cpp:2130-2137).  Each update rebuilds its entry with the same float
// operations, (int)(p0 + p1p0 * k), so results stay bit-identical while a warp's 32 lookups fall on
// ~10 consecutive 8-byte pairs (no bank conflicts) and the table is 8x smaller.  With
// y = fl_rz(fx + 2^23) = 2^23 + floor(fx):  fl = y - 2^23 = floor(fx),
// z = fl_rz(fl/16 + 2^23) = 2^23 + j,  k = fl - 16 j  -- all exact in FP32 for 0 <= fx < 2^23.
// Per-view record of the pair-table kernel.
struct PairMeta {
    int w0;      // window start (pair index)
    int nwin;    // window length in pairs
    int a, b;    // in-table part [a, b) of the window
    int fast;    // 1: every fx of the tile is >= 0
    int pad0, pad1, pad2;
};

template <int WX, int WY, int RX, int RY, int VC>
struct PairCfg {
    static constexpr int NT = 32 * WX * WY;
    static constexpr int GX = 8 * WX, GY = 4 * WY;
    static constexpr int TX = GX * RX, TY = GY * RY;
    // detector-pixel span of a tile: sqrt((TX-1)^2 + (TY-1)^2) + margins + even alignment
    static constexpr int WINJ = ((isqrt_ceil((TX - 1) * (TX - 1) + (TY - 1) * (TY - 1)) + 8) + 3) / 4 * 4;
    static constexpr size_t SMEM = (size_t)2 * VC * WINJ * 8 + (size_t)3 * VC * (TX + TY) * 4 + (size_t)3 * VC * 32 + 16;
};

template <int WX, int WY, int RX, int RY, int VC, int MINB, bool CHECKED>
__global__ void __launch_bounds__(32 * WX * WY, MINB) k_bp_pair(BackprojLaunch p) {
    using Cfg = PairCfg<WX, WY, RX, RY, VC>;
    constexpr int NT = Cfg::NT, TX = Cfg::TX, TY = Cfg::TY, WINJ = Cfg::WINJ;
    extern __shared__ __align__(128) int smi[];
    float2* win = reinterpret_cast<float2*>(smi);                       // [2][VC][WINJ]
    float* xs = reinterpret_cast<float*>(win + 2 * VC * WINJ);          // [3][VC][TX]
    float* ys = xs + 3 * VC * TX;                                       // [3][VC][TY]
    PairMeta* meta = reinterpret_cast<PairMeta*>(ys + 3 * VC * TY);     // [3][VC]
    uint64_t* bars = reinterpret_cast<uint64_t*>(meta + 3 * VC);        // [2]

    const int ixdimp = p.ixdimp;
    const int tiles_x = (ixdimp + TX - 1) / TX;
    const int X0 = (blockIdx.x % tiles_x) * TX;
    const int Y0 = (blockIdx.x / tiles_x) * TY;
    const int slice = blockIdx.y;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx = (warp % WX) * 8 + (lane & 7);
    const int ty = (warp / WX) * 4 + (lane >> 3);
    const float2* tab = reinterpret_cast<const float2*>(p.table + (size_t)slice * p.slice_table_stride);
    const int npairs = (ixdimp + 1) & ~1;   // the filter writes a zero pair at j = ixdimp when odd
    const int nviews = p.nviews;
    const int nchunks = (nviews + VC - 1) / VC;
    unsigned viol = 0;

    if (tid == 0) {
        mbar_init(smem_u32(&bars[0]), 1);
        mbar_init(smem_u32(&bars[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    auto prepare = [&](int c, int ms) {
        const int v0 = c * VC;
        if (tid < VC && v0 + tid < nviews) {
            const float4 g = __ldg(p.geom + (size_t)slice * p.geom_slice_stride + v0 + tid);
            float lo = 3.0e38f, hi = -3.0e38f;
#pragma unroll
            for (int cy = 0; cy < 2; cy++) {
                const float fy = faddr(fmulr((float)(Y0 + cy * (TY - 1)), g.y), g.z);
#pragma unroll
                for (int cx = 0; cx < 2; cx++) {
                    const float fx = faddr(fmulr((float)(X0 + cx * (TX - 1)), g.x), fy);
                    lo = fminf(lo, fx);
                    hi = fmaxf(hi, fx);
                }
            }
            const int ilo = (int)floorf(lo) - 2;       // index range [ilo, ihi)
            const int ihi = (int)floorf(hi) + 3;
            PairMeta m;
            m.w0 = (ilo >> 4) & ~1;                    // first pair (even, floor division)
            const int jhi = (((ihi - 1) >> 4) + 2) & ~1;
            m.nwin = min(jhi - m.w0, WINJ);
            m.a = max(m.w0, 0);
            m.b = min(m.w0 + m.nwin, npairs);
            m.fast = (lo >= 2.0f) ? 1 : 0;
            m.pad0 = m.pad1 = m.pad2 = 0;
            meta[ms * VC + tid] = m;
        }
        for (int e = tid; e < VC * (TX + TY); e += NT) {
            const int vv = e / (TX + TY), w = e - vv * (TX + TY);
            if (v0 + vv >= nviews) continue;
            const float4 g = __ldg(p.geom + (size_t)slice * p.geom_slice_stride + v0 + vv);
            if (w < TX) {
                const int t = w / RX, c = w - t * RX;
                xs[(ms * VC + vv) * TX + w] = fmulr((float)(X0 + t + Cfg::GX * c), g.x);
            } else {
                const int w2 = w - TX, t = w2 / RY, r = w2 - t * RY;
                ys[(ms * VC + vv) * TY + w2] = faddr(fmulr((float)(Y0 + t + Cfg::GY * r), g.y), g.z);
            }
        }
    };
    auto stage = [&](int c, int ms, int wb) {
        const int v0 = c * VC;
        const int nv = min(VC, nviews - v0);
        if (tid == 0) {
            unsigned bytes = 0;
            for (int vv = 0; vv < nv; vv++) {
                const PairMeta m = meta[ms * VC + vv];
                if (m.b > m.a) bytes += 8u * (unsigned)(m.b - m.a);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const unsigned bar = smem_u32(&bars[wb]);
            mbar_arrive_expect_tx(bar, bytes);
            for (int vv = 0; vv < nv; vv++) {
                const PairMeta m = meta[ms * VC + vv];
                if (m.b <= m.a) continue;
                const float2* src = tab + (size_t)(v0 + vv) * (p.table_stride / 2) + m.a;
                const unsigned dst = smem_u32(win + (wb * VC + vv) * WINJ + (m.a - m.w0));
                tma_bulk_g2s(dst, src, 8u * (unsigned)(m.b - m.a), bar);
            }
        }
        for (int vv = 0; vv < nv; vv++) {
            const PairMeta m = meta[ms * VC + vv];
            float4* w4 = reinterpret_cast<float4*>(win + (wb * VC + vv) * WINJ);   // 2 pairs per float4
            const int za = (m.b > m.a) ? (m.a - m.w0) >> 1 : m.nwin >> 1;
            const int zb = (m.b > m.a) ? (m.b - m.w0) >> 1 : m.nwin >> 1;
            for (int e = tid; e < za; e += NT) w4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int e = zb + tid; e < ((m.nwin + 1) >> 1); e += NT) w4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };

    int acc[RY][RX];
#pragma unroll
    for (int r = 0; r < RY; r++)
#pragma unroll
        for (int c = 0; c < RX; c++) acc[r][c] = 0;

    prepare(0, 0);
    if (nchunks > 1) prepare(1, 1);
    __syncthreads();
    stage(0, 0, 0);
    for (int k = 0; k < nchunks; k++) {
        const int wb = k & 1, ms = k % 3;
        if (k + 1 < nchunks) stage(k + 1, (k + 1) % 3, wb ^ 1);
        if (k + 2 < nchunks) prepare(k + 2, (k + 2) % 3);
        const bool ok = mbar_wait_bounded(smem_u32(&bars[wb]), (unsigned)(k >> 1) & 1u);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(&g_kernel_status, 1u);
            mbar_wait_bounded(smem_u32(&bars[wb]), (unsigned)(k >> 1) & 1u);
            if (k + 1 < nchunks) mbar_wait_bounded(smem_u32(&bars[wb ^ 1]), (unsigned)((k + 1) >> 1) & 1u);
            return;
        }
        const int nv = min(VC, nviews - k * VC);
        for (int vv = 0; vv < nv; vv++) {
            const PairMeta m = meta[ms * VC + vv];
            float xv[RX], yv[RY];
#pragma unroll
            for (int c4 = 0; c4 < RX; c4 += 4) {
                const float4 t4 = *reinterpret_cast<const float4*>(xs + (ms * VC + vv) * TX + tx * RX + c4);
                xv[c4] = t4.x; xv[c4 + 1] = t4.y; xv[c4 + 2] = t4.z; xv[c4 + 3] = t4.w;
            }
#pragma unroll
            for (int r4 = 0; r4 < RY; r4 += 4) {
                const float4 t4 = *reinterpret_cast<const float4*>(ys + (ms * VC + vv) * TY + ty * RY + r4);
                yv[r4] = t4.x; yv[r4 + 1] = t4.y; yv[r4 + 2] = t4.z; yv[r4 + 3] = t4.w;
            }
            const float2* wv = win + (wb * VC + vv) * WINJ;
            const unsigned wbase = smem_u32(wv) - 8u * (unsigned)m.w0;
            if (m.fast) {
                const unsigned base = wbase - 8u * kMagicBits;
#pragma unroll
                for (int r = 0; r < RY; r++)
#pragma unroll
                    for (int c = 0; c < RX; c++) {
                        const float fx = faddr(xv[c], yv[r]);
                        const float y = __fadd_rz(fx, 8388608.0f);
                        const float fl = __fsub_rn(y, 8388608.0f);            // floor(fx)
                        const float z = __fmaf_rz(fl, 0.0625f, 8388608.0f);   // 2^23 + j
                        const float jf = __fsub_rn(z, 8388608.0f);
                        const float kf = __fmaf_rn(-16.0f, jf, fl);            // k, exact
                        const unsigned zb = __float_as_uint(z);
                        if (CHECKED) {
                            const int j = (int)(zb - kMagicBits);
                            if (fx < 0.0f || j < m.w0 || j >= m.w0 + m.nwin) { viol++; continue; }
                        }
                        float2 pr;
                        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(pr.x), "=f"(pr.y) : "r"(base + 8u * zb));
                        acc[r][c] += __float2int_rz(faddr(pr.x, fmulr(pr.y, kf)));
                    }
            } else {
#pragma unroll
                for (int r = 0; r < RY; r++)
#pragma unroll
                    for (int c = 0; c < RX; c++) {
                        const float fx = faddr(xv[c], yv[r]);
                        const int ix = __float2int_rz(fx);        // the reference's (int)fx
                        const int j = ix >> 4;                    // floor division
                        const float kf = (float)(ix & 15);
                        if (CHECKED) {
                            if (j < m.w0 || j >= m.w0 + m.nwin) { viol++; continue; }
                        }
                        float2 pr;
                        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(pr.x), "=f"(pr.y) : "r"(wbase + 8u * (unsigned)j));
                        acc[r][c] += __float2int_rz(faddr(pr.x, fmulr(pr.y, kf)));
                    }
            }
        }
        __syncthreads();
    }
    if (CHECKED && viol) atomicAdd(p.status_counter, viol);

    int* out = static_cast<int*>(p.out) + (size_t)slice * p.out_slice_stride;
#pragma unroll
    for (int r = 0; r < RY; r++) {
        const int y = Y0 + ty + Cfg::GY * r;
        if (y >= ixdimp) continue;
#pragma unroll
        for (int c = 0; c < RX; c++) {
            const int x = X0 + tx + Cfg::GX * c;
            if (x < ixdimp) out[(size_t)y * ixdimp + x] = acc[r][c];
        }
    }
}

// ---- configuration ---------------------------------------------------------------------------
// Table format (RvSetBackprojectionVariant's second argument, or RV_BP_FORMAT) and variant
// (first argument, or RV_BP_VARIANT):
//   int tables (format 0 dense / 1 padded), 32 px per thread unless noted:
//     0: 128x128 tile, 512 threads, 8 views/chunk   1: 64x64, 256 threads, 16 px/thread
//     2: 128x128, 512 threads, 4 views/chunk
//     3: 64x64, 256 threads, 16 px/thread, 4 views/chunk, 4 CTAs/SM
//     4: 128x64, 512 threads, 16 px/thread, 4 views/chunk, 2 CTAs/SM
//     5: 64x128, 256 threads, 32 px/thread, 4 views/chunk, 2 CTAs/SM
//     6, 7, 8: variants 3, 0, 4 with the column/row products formed in registers (OTF)
//     9, 10, 11: 64x64 OTF without block barriers (warp-decoupled pipeline) with 3x3, 4x2, 2x4
//        buffers x views per chunk;  12: 128x128, 512 threads, 3 buffers x 4 views;
//     13: 128x64, 512 threads, 2 x 4;  14, 15: 64x64, 2 buffers x 5 / 6 views, 3 CTAs/SM
//     16: 64x64, 8 consumer warps + 1 producer warp, ray-aligned lane footprints (shear steps
//         of 1/12), 2 buffers x 6 views, 3 CTAs/SM;  17: the same with compact 8x4 lane blocks,
//         2 buffers x 4 views, 4 CTAs/SM;  18: variant 16's layout over slice pairs (two
//         slices sharing the geometry per CTA: one index per pixel and view, two gathers),
//         2 buffers x 4 views x 2 slices, 2 CTAs/SM;  19: variant 18 with 16 consumer warps
//         (8 pixels x 2 slices per thread);  20: four slices per CTA sharing the index, 16
//         consumer warps (8 pixels x 4 slices per thread), 2 buffers x 4 views x 4 slices, 1 CTA/SM
//     21: three slices per CTA sharing the index (16 pixels x 3 slices per thread), 2 buffers x
//         3 views x 3 slices, 2 CTAs/SM; the rest of a stack as slice pairs (the default)
//   pair tables (format 2):
//     0: 128x128 tile, 512 threads, 16 views/chunk  1: 64x128, 256 threads, 2 CTAs/SM
//     2: 128x64, 512 threads, 16 px/thread, 2 CTAs/SM
static int env_int(const char* name, int dflt) {
    const char* e = getenv(name);
    return e ? atoi(e) : dflt;
}
static int g_variant = -1, g_fmt = -1;
static void load_defaults() {
    if (g_variant < 0) g_variant = env_int("RV_BP_VARIANT", 21);
    if (g_fmt < 0) g_fmt = env_int("RV_BP_FORMAT", kTabInt16);
}
int ref_table_fmt() {
    load_defaults();
    return g_fmt;
}
// The default layout's regime (NQ = 12) of a view, tagged for regime_of: an orientation bit and
// the shear k = rint(12 t), t = -fcos/fsin or -fsin/fcos, whichever has |t| <= 1.  Any value would
// give the same slices; the tag only spares every consumer thread the division per chunk.
float ray_regime_tag(float gc, float gs) {
    constexpr int NQ = 12;
    const bool h = fabsf(gs) > fabsf(gc);
    const float den = h ? gs : gc;
    int k = 0;
    if (den != 0.0f) {
        const float t = (h ? -gc : -gs) / den;
        k = (int)lrintf(t * (float)NQ);
        k = k < -NQ ? -NQ : (k > NQ ? NQ : k);
    }
    const unsigned r = (h ? 1u : 0u) | ((unsigned)(k + NQ) << 1);
    const unsigned w = kRegimeTag | ((unsigned)NQ << 16) | r;
    float f;
    memcpy(&f, &w, sizeof f);
    return f;
}

long long ref_table_stride(int ixdimp, int fmt) {
    if (fmt == kTabPair) return 2LL * ((ixdimp + 1) & ~1);   // floats, pairs rounded to an even count
    if (fmt == kTabInt17) return ((long long)17 * ixdimp + 15) & ~15LL;
    return 16LL * ixdimp;
}

// Validation mode: window violations counted by the checked kernels into a __device__ word,
// whose address is resolved at each checked launch (so a device reset never leaves a stale one).
static int g_checked = 0;
__device__ unsigned int g_window_violation_count = 0;
static unsigned long long g_violations = 0;

template <typename K>
static cudaError_t launch_k(K kern, dim3 grid, int nt, size_t smem, const BackprojLaunch& p, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, nt, smem, s>>>(p);
    t_bp_launches++;
    return cudaGetLastError();
}

template <int WX, int WY, int RX, int RY, int VC, int PAD, int MINB, int OTF = 0>
static cudaError_t go_bp(const BackprojLaunch& p, cudaStream_t s, bool checked) {
    using Cfg = BpCfg<WX, WY, RX, RY, VC, PAD, OTF>;
    const int tiles = ((p.ixdimp + Cfg::TX - 1) / Cfg::TX) * ((p.ixdimp + Cfg::TY - 1) / Cfg::TY);
    dim3 grid(tiles, p.nslices);
    if (checked)
        return launch_k(k_bp_ref<WX, WY, RX, RY, VC, PAD, MINB, OTF, true>, grid, Cfg::NT, Cfg::SMEM, p, s);
    return launch_k(k_bp_ref<WX, WY, RX, RY, VC, PAD, MINB, OTF, false>, grid, Cfg::NT, Cfg::SMEM, p, s);
}

template <int WX, int WY, int RX, int RY, int VC, int NB, int PAD, int MINB>
static cudaError_t go_pipe(const BackprojLaunch& p, cudaStream_t s, bool checked) {
    using Cfg = PipeCfg<WX, WY, RX, RY, VC, NB, PAD>;
    const int tiles = ((p.ixdimp + Cfg::TX - 1) / Cfg::TX) * ((p.ixdimp + Cfg::TY - 1) / Cfg::TY);
    dim3 grid(tiles, p.nslices);
    if (checked)
        return launch_k(k_bp_ref_pipe<WX, WY, RX, RY, VC, NB, PAD, MINB, true>, grid, Cfg::NT, Cfg::SMEM, p, s);
    return launch_k(k_bp_ref_pipe<WX, WY, RX, RY, VC, NB, PAD, MINB, false>, grid, Cfg::NT, Cfg::SMEM, p, s);
}

// Number of view groups for a launch of `ctas` tile CTAs on `slots` resident CTA slots: the
// last wave of a small launch (one slice: 1024 tiles on 456 slots) would run mostly empty, so
// the views are split into g groups whose partial sums are added into the slice, choosing g
// (1..8, at least 16 views per group) for the least time ceil(ctas g / slots) / g.
static int view_groups(long long ctas, int slots, int nviews) {
    if (slots <= 0 || ctas <= 0 || ctas >= 8LL * slots) return 1;
    int best = 1;
    double best_t = (double)((ctas + slots - 1) / slots);
    for (int g = 2; g <= 8 && nviews / g >= 16; g++) {
        const double t = (double)((ctas * g + slots - 1) / slots) / g;
        if (t < 0.97 * best_t) {
            best_t = t;
            best = g;
        }
    }
    return best;
}

template <int VC, int NB, int PAD, int NQ, int MINB, int NS = 1, int CW = 8>
static cudaError_t go_ws_rows(const BackprojLaunch& p, cudaStream_t s, bool checked, int slice0, int rows) {
    using Cfg = WsCfg<VC, NB, PAD, NS, CW>;
    const int tiles = ((p.ixdimp + 63) / 64) * ((p.ixdimp + 63) / 64);
    auto kern = checked ? k_bp_ref_ws<VC, NB, PAD, NQ, MINB, true, NS, CW> : k_bp_ref_ws<VC, NB, PAD, NQ, MINB, false, NS, CW>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Cfg::NT, Cfg::SMEM) != cudaSuccess) per_sm = 0;
    const int groups = view_groups((long long)tiles * rows, sms * per_sm, p.nviews);
    if (groups > 1) {   // the groups add into zeroed slices
        e = cudaMemsetAsync(static_cast<int*>(p.out) + (size_t)slice0 * p.out_slice_stride, 0,
                            (size_t)rows * NS * p.out_slice_stride * sizeof(int), s);
        if (e != cudaSuccess) return e;
    }
    kern<<<dim3(tiles, rows, groups), Cfg::NT, Cfg::SMEM, s>>>(p, slice0);
    t_bp_launches++;
    return cudaGetLastError();
}

template <int VC, int NB, int PAD, int NQ, int MINB>
static cudaError_t go_ws(const BackprojLaunch& p, cudaStream_t s, bool checked) {
    return go_ws_rows<VC, NB, PAD, NQ, MINB>(p, s, checked, 0, p.nslices);
}

// slice pairs (two slices per CTA sharing the index arithmetic) when the slices share the
// geometry; an odd last slice, or per-slice geometry, runs one slice per CTA (variant 16's form)
template <int VC, int NB, int PAD, int NQ, int MINB, int CW = 8>
static cudaError_t go_ws_pairs(const BackprojLaunch& p, cudaStream_t s, bool checked) {
    if (p.geom_slice_stride != 0 || p.nslices < 2) return go_ws_rows<6, 2, PAD, 12, 3>(p, s, checked, 0, p.nslices);
    cudaError_t e = go_ws_rows<VC, NB, PAD, NQ, MINB, 2, CW>(p, s, checked, 0, p.nslices / 2);
    if (e == cudaSuccess && (p.nslices & 1)) e = go_ws_rows<6, 2, PAD, 12, 3>(p, s, checked, p.nslices - 1, 1);
    return e;
}

// groups of four slices per CTA (one index per pixel and view, four gathers), then pairs and a
// single slice for the rest; per-slice geometry runs one slice per CTA
template <int VC, int NB, int PAD, int NQ, int MINB, int CW>
static cudaError_t go_ws_quads(const BackprojLaunch& p, cudaStream_t s, bool checked) {
    if (p.geom_slice_stride != 0 || p.nslices < 4) return go_ws_pairs<4, 2, PAD, 12, 2>(p, s, checked);
    const int q4 = p.nslices / 4;
    cudaError_t e = go_ws_rows<VC, NB, PAD, NQ, MINB, 4, CW>(p, s, checked, 0, q4);
    const int rest = p.nslices - 4 * q4;
    if (e == cudaSuccess && rest >= 2) e = go_ws_rows<4, 2, PAD, 12, 2, 2>(p, s, checked, 4 * q4, 1);
    if (e == cudaSuccess && (rest & 1)) e = go_ws_rows<6, 2, PAD, 12, 3>(p, s, checked, p.nslices - 1, 1);
    return e;
}

// groups of three slices per CTA (one index per pixel and view, three gathers), the rest as
// slice pairs: n = 3t, 3t + 2 (one pair) or 3(t - 1) + 4 (two pairs); fewer than three slices,
// or per-slice geometry, go to the pair form
template <int VC, int NB, int PAD, int NQ, int MINB, int CW = 8>
static cudaError_t go_ws_triples(const BackprojLaunch& p, cudaStream_t s, bool checked) {
    if (p.geom_slice_stride != 0 || p.nslices < 3) return go_ws_pairs<4, 2, PAD, 12, 2>(p, s, checked);
    int t3 = p.nslices / 3;
    if (p.nslices % 3 == 1) t3--;
    cudaError_t e = t3 > 0 ? go_ws_rows<VC, NB, PAD, NQ, MINB, 3, CW>(p, s, checked, 0, t3) : cudaSuccess;
    const int rest = p.nslices - 3 * t3;
    if (e == cudaSuccess && rest >= 2) e = go_ws_rows<4, 2, PAD, 12, 2, 2>(p, s, checked, 3 * t3, rest / 2);
    if (e == cudaSuccess && (rest & 1)) e = go_ws_rows<6, 2, PAD, 12, 3>(p, s, checked, p.nslices - 1, 1);
    return e;
}

template <int WX, int WY, int RX, int RY, int VC, int MINB>
static cudaError_t go_pair(const BackprojLaunch& p, cudaStream_t s, bool checked) {
    using Cfg = PairCfg<WX, WY, RX, RY, VC>;
    const int tiles = ((p.ixdimp + Cfg::TX - 1) / Cfg::TX) * ((p.ixdimp + Cfg::TY - 1) / Cfg::TY);
    dim3 grid(tiles, p.nslices);
    if (checked) return launch_k(k_bp_pair<WX, WY, RX, RY, VC, MINB, true>, grid, Cfg::NT, Cfg::SMEM, p, s);
    return launch_k(k_bp_pair<WX, WY, RX, RY, VC, MINB, false>, grid, Cfg::NT, Cfg::SMEM, p, s);
}

template <int PAD>
static cudaError_t dispatch_bp(const BackprojLaunch& p, cudaStream_t s, bool checked, int variant) {
    switch (variant) {
    case 1: return go_bp<2, 4, 4, 4, 8, PAD, 1>(p, s, checked);
    case 2: return go_bp<4, 4, 4, 8, 4, PAD, 1>(p, s, checked);
    case 3: return go_bp<2, 4, 4, 4, 4, PAD, 4>(p, s, checked);
    case 4: return go_bp<4, 4, 4, 4, 4, PAD, 2>(p, s, checked);
    case 5: return go_bp<2, 4, 4, 8, 4, PAD, 2>(p, s, checked);
    case 6: return go_bp<2, 4, 4, 4, 4, PAD, 4, 1>(p, s, checked);
    case 7: return go_bp<4, 4, 4, 8, 8, PAD, 1, 1>(p, s, checked);
    case 8: return go_bp<4, 4, 4, 4, 4, PAD, 2, 1>(p, s, checked);
    case 9: return go_pipe<2, 4, 4, 4, 3, 3, PAD, 4>(p, s, checked);
    case 10: return go_pipe<2, 4, 4, 4, 2, 4, PAD, 4>(p, s, checked);
    case 11: return go_pipe<2, 4, 4, 4, 4, 2, PAD, 4>(p, s, checked);
    case 12: return go_pipe<4, 4, 4, 8, 4, 3, PAD, 1>(p, s, checked);
    case 13: return go_pipe<4, 4, 4, 4, 4, 2, PAD, 2>(p, s, checked);
    case 14: return go_pipe<2, 4, 4, 4, 5, 2, PAD, 3>(p, s, checked);
    case 15: return go_pipe<2, 4, 4, 4, 6, 2, PAD, 3>(p, s, checked);
    case 16: return go_ws<6, 2, PAD, 12, 3>(p, s, checked);
    case 17: return go_ws<4, 2, PAD, 0, 4>(p, s, checked);
    case 18: return go_ws_pairs<4, 2, PAD, 12, 2>(p, s, checked);
    case 19: return go_ws_pairs<4, 2, PAD, 8, 2, 16>(p, s, checked);
    case 21: return go_ws_triples<3, 2, PAD, 12, 2>(p, s, checked);
    case 20: return go_ws_quads<4, 2, PAD, 8, 1, 16>(p, s, checked);
    default: return go_bp<4, 4, 4, 8, 8, PAD, 1>(p, s, checked);
    }
}

static cudaError_t dispatch_pair(const BackprojLaunch& p, cudaStream_t s, bool checked, int variant) {
    switch (variant) {
    case 1: return go_pair<2, 4, 4, 8, 16, 2>(p, s, checked);
    case 2: case 4: case 5: case 8: return go_pair<4, 4, 4, 4, 16, 2>(p, s, checked);
    case 3: case 6: case 9: case 10: case 11: case 14: case 15: return go_pair<2, 4, 4, 4, 8, 4>(p, s, checked);
    case 13: return go_pair<4, 4, 4, 4, 16, 2>(p, s, checked);
    default: return go_pair<4, 4, 4, 8, 16, 1>(p, s, checked);
    }
}

// Persistent launcher for the batched queue: the tile shape of the selected int-table variant
// (variants 0/2 -> 128x128, 4 -> 128x64, else 64x64), one grid of (SMs x resident CTAs).
template <int WX, int WY, int RX, int RY, int VC, int PAD, int MINB, int OTF = 0>
static cudaError_t go_persistent(const TileJob* jobs, int njobs, unsigned* counter, cudaStream_t s) {
    using Cfg = BpCfg<WX, WY, RX, RY, VC, PAD, OTF>;
    auto kern = k_bp_ref_persistent<WX, WY, RX, RY, VC, PAD, MINB, OTF>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Cfg::NT, Cfg::SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int grid = sms * per_sm;
    if (grid > njobs) grid = njobs;
    if (grid < 1) return cudaSuccess;
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(jobs, njobs, counter);
    return cudaGetLastError();
}

template <int WX, int WY, int RX, int RY, int VC, int NB, int PAD, int MINB>
static cudaError_t go_pipe_persistent(const TileJob* jobs, int njobs, unsigned* counter, cudaStream_t s) {
    using Cfg = PipeCfg<WX, WY, RX, RY, VC, NB, PAD>;
    auto kern = k_bp_ref_pipe_persistent<WX, WY, RX, RY, VC, NB, PAD, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Cfg::NT, Cfg::SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int grid = sms * per_sm;
    if (grid > njobs) grid = njobs;
    if (grid < 1) return cudaSuccess;
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(jobs, njobs, counter);
    return cudaGetLastError();
}

template <int VC, int NB, int PAD, int NQ, int MINB, int NSL = 1, int CW = 8>
static cudaError_t go_ws_persistent(const TileJob* jobs, int njobs, unsigned* counter, cudaStream_t s) {
    using Cfg = WsCfg<VC, NB, PAD, NSL, CW>;
    auto kern = k_bp_ref_ws_persistent<VC, NB, PAD, NQ, MINB, NSL, CW>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::SMEM);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Cfg::NT, Cfg::SMEM);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int grid = sms * per_sm;
    if (grid > njobs) grid = njobs;
    if (grid < 1) return cudaSuccess;
    kern<<<grid, Cfg::NT, Cfg::SMEM, s>>>(jobs, njobs, counter);
    return cudaGetLastError();
}

static void persistent_shape(int variant, int* tx, int* ty) {
    switch (variant) {
    case 0: case 2: case 7: case 12: *tx = 128; *ty = 128; break;
    case 4: case 8: case 13: *tx = 128; *ty = 64; break;
    case 5: *tx = 64; *ty = 128; break;
    default: *tx = 64; *ty = 64; break;
    }
}

void persistent_tile_xy(int variant, int* tx, int* ty) { persistent_shape(variant, tx, ty); }

template <int PAD>
static cudaError_t dispatch_persistent(const TileJob* jobs, int njobs, unsigned* counter, cudaStream_t s, int variant) {
    switch (variant) {
    case 0: return go_persistent<4, 4, 4, 8, 8, PAD, 1>(jobs, njobs, counter, s);
    case 2: return go_persistent<4, 4, 4, 8, 4, PAD, 1>(jobs, njobs, counter, s);
    case 4: return go_persistent<4, 4, 4, 4, 4, PAD, 2>(jobs, njobs, counter, s);
    case 5: return go_persistent<2, 4, 4, 8, 4, PAD, 2>(jobs, njobs, counter, s);
    case 1: return go_persistent<2, 4, 4, 4, 8, PAD, 1>(jobs, njobs, counter, s);
    case 6: return go_persistent<2, 4, 4, 4, 4, PAD, 4, 1>(jobs, njobs, counter, s);
    case 7: return go_persistent<4, 4, 4, 8, 8, PAD, 1, 1>(jobs, njobs, counter, s);
    case 8: return go_persistent<4, 4, 4, 4, 4, PAD, 2, 1>(jobs, njobs, counter, s);
    case 9: return go_pipe_persistent<2, 4, 4, 4, 3, 3, PAD, 4>(jobs, njobs, counter, s);
    case 10: return go_pipe_persistent<2, 4, 4, 4, 2, 4, PAD, 4>(jobs, njobs, counter, s);
    case 11: return go_pipe_persistent<2, 4, 4, 4, 4, 2, PAD, 4>(jobs, njobs, counter, s);
    case 12: return go_pipe_persistent<4, 4, 4, 8, 4, 3, PAD, 1>(jobs, njobs, counter, s);
    case 13: return go_pipe_persistent<4, 4, 4, 4, 4, 2, PAD, 2>(jobs, njobs, counter, s);
    case 14: return go_pipe_persistent<2, 4, 4, 4, 5, 2, PAD, 3>(jobs, njobs, counter, s);
    case 15: return go_pipe_persistent<2, 4, 4, 4, 6, 2, PAD, 3>(jobs, njobs, counter, s);
    case 16: return go_ws_persistent<6, 2, PAD, 12, 3>(jobs, njobs, counter, s);
    case 18: return go_ws_persistent<4, 2, PAD, 12, 2, 2>(jobs, njobs, counter, s);
    case 19: return go_ws_persistent<4, 2, PAD, 8, 2, 2, 16>(jobs, njobs, counter, s);
    case 20: return go_ws_persistent<4, 2, PAD, 12, 2, 2>(jobs, njobs, counter, s);
    case 21: return go_ws_persistent<3, 2, PAD, 12, 2, 3>(jobs, njobs, counter, s);   // triple and pair jobs
    case 17: return go_ws_persistent<4, 2, PAD, 0, 4>(jobs, njobs, counter, s);
    default: return go_persistent<2, 4, 4, 4, 4, PAD, 4>(jobs, njobs, counter, s);
    }
}

cudaError_t launch_bp_ref_persistent(const TileJob* d_jobs, int njobs, unsigned* d_counter, int table_fmt,
                                     int variant, cudaStream_t s) {
    if (table_fmt == kTabPair) return cudaErrorInvalidValue;   // queue tables are int tables
    return table_fmt == kTabInt17 ? dispatch_persistent<1>(d_jobs, njobs, d_counter, s, variant)
                                  : dispatch_persistent<0>(d_jobs, njobs, d_counter, s, variant);
}
int default_variant() {
    load_defaults();
    return g_variant;
}
int take_backproject_launches() {
    const int n = t_bp_launches;
    t_bp_launches = 0;
    return n;
}

cudaError_t launch_bp_ref(const BackprojLaunch& pin, cudaStream_t s) {
    load_defaults();
    return launch_bp_ref_variant(pin, s, g_variant);
}

cudaError_t launch_bp_ref_variant(const BackprojLaunch& pin, cudaStream_t s, int variant) {
    BackprojLaunch p = pin;
    load_defaults();
    const bool checked = g_checked != 0;
    unsigned int* counter = nullptr;
    if (checked) {
        cudaError_t e = cudaGetSymbolAddress((void**)&counter, g_window_violation_count);
        if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess) return e;
        p.status_counter = counter;
    }
    cudaError_t e;
    if (p.table_fmt == kTabPair) e = dispatch_pair(p, s, checked, variant);
    else if (p.table_fmt == kTabInt17) e = dispatch_bp<1>(p, s, checked, variant);
    else e = dispatch_bp<0>(p, s, checked, variant);
    if (checked && e == cudaSuccess) {
        unsigned int v = 0;
        e = cudaMemcpyAsync(&v, counter, sizeof(v), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        g_violations += v;
    }
    return e;
}

unsigned int take_kernel_status(cudaStream_t s) {
    unsigned int v = 0, zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_kernel_status, sizeof(v), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return kStatusUnreadable;
    if (cudaStreamSynchronize(s) != cudaSuccess) return kStatusUnreadable;
    if (v) {
        if (cudaMemcpyToSymbolAsync(g_kernel_status, &zero, sizeof(zero), 0, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            v |= kStatusUnreadable;
    }
    return v;
}
const char* kernel_status_text(unsigned int status) {
    if (status & kStatusUnreadable) return "the kernel status word could not be read (copy or synchronisation failed)";
    if (status & kStatusWaitRanOut) return "a bounded wait for a table copy ran out";
    return "no error";
}

}  // namespace rv

namespace rv {
// Failure-detection check: one CTA waits on an mbarrier that nothing completes, with the same
// bounded wait as the kernels (2^LOG2 tries of at most ~1 us), then reports the timeout through
// g_kernel_status and returns; the context stays usable.
template <int LOG2>
__global__ void k_wait_runs_out(unsigned* tries_out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bar), 1);   // one arrival expected, none comes
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded<LOG2>(smem_u32(&bar), 0u));
    if (!ok && threadIdx.x == 0) {
        atomicOr(&g_kernel_status, 1u);
        *tries_out = 1u << LOG2;
    }
}
}  // namespace rv

// Runs the bounded-wait check (log2_tries 8..16) and returns RV_ERR_KERNEL_STATUS when the wait
// ran out as it must, after clearing the status; *elapsed_ms gets the kernel's duration.
extern "C" int RvTestBoundedWait(int log2_tries, double* elapsed_ms) {
    if (log2_tries < 8 || log2_tries > 16) return RV_ERR_BAD_ARGUMENT;
    unsigned* d_tries = nullptr;
    if (cudaMalloc(&d_tries, sizeof(unsigned)) != cudaSuccess) return RV_ERR_DEVICE_OOM;
    cudaMemset(d_tries, 0, sizeof(unsigned));
    rv::take_kernel_status(0);   // start from a clear status
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, 0);
    switch (log2_tries) {
    case 8: rv::k_wait_runs_out<8><<<1, 32>>>(d_tries); break;
    case 12: rv::k_wait_runs_out<12><<<1, 32>>>(d_tries); break;
    default: rv::k_wait_runs_out<16><<<1, 32>>>(d_tries); break;
    }
    cudaEventRecord(e1, 0);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (elapsed_ms) *elapsed_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_tries);
    if (e != cudaSuccess) return RV_ERR_LAUNCH;
    return rv::take_kernel_status(0) ? RV_ERR_KERNEL_STATUS : 0;
}

extern "C" int RvSetCheckedBackprojection(int enable) {
    rv::g_checked = enable ? 1 : 0;
    rv::g_violations = 0;
    return 0;
}
extern "C" unsigned long long RvGetWindowViolations(void) { return rv::g_violations; }

extern "C" int RvSetBackprojectionVariant(int variant, int format) {
    if (variant < 0 || variant > 21 || format < 0 || format > 2) return RV_ERR_BAD_ARGUMENT;
    rv::g_variant = variant;
    rv::g_fmt = format;
    return 0;
}
extern "C" int RvGetBackprojectionVariant(int* variant, int* format) {
    rv::load_defaults();
    if (variant) *variant = rv::g_variant;
    if (format) *format = rv::g_fmt;
    return 0;
}
