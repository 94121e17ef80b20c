// R9: the post-processing that CGazoDoc::DeconvBackProj applies to a finished int32 slice
// (source/gazoDoc.cpp:3993-4021): global min/max (max starts at 0), a circular mask around the
// detector-pixel centre and the linear map to 0..65534, in float, exactly as the reference.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include "rv_internal.h"

namespace rv {

__global__ void k_minmax(const int* __restrict__ in, long long n, int* mm) {
    // mm[0] = min, mm[1] = max of one slice (grid.y = slice)
    const int* s = in + (long long)blockIdx.y * n;
    int lo = INT_MAX, hi = 0;   // the reference starts imax at 0 (source/gazoDoc.cpp:3993)
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int v = s[i];
        lo = min(lo, v);
        hi = max(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __shared__ int slo[32], shi[32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        slo[w] = lo;
        shi[w] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) {
            lo = min(lo, slo[k]);
            hi = max(hi, shi[k]);
        }
        atomicMin(&mm[2 * blockIdx.y], lo);
        atomicMax(&mm[2 * blockIdx.y + 1], hi);
    }
}

__global__ void k_rescale(int* __restrict__ io, uint16_t* __restrict__ out16, int ixdimp, int irad2, const int* mm) {
    const int y = blockIdx.y, slice = blockIdx.z;
    const long long n = (long long)ixdimp * ixdimp;
    int imin = mm[2 * slice], imax = mm[2 * slice + 1];
    if (imin == imax) imax++;
    const float den = (float)(imax - imin);
    const int ixdimh = ixdimp / 2;
    const int i2 = (y - ixdimh) * (y - ixdimh);
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < ixdimp; x += gridDim.x * blockDim.x) {
        const long long idx = (long long)slice * n + (long long)y * ixdimp + x;
        const int j2 = x - ixdimh;
        int v = 0;
        if (i2 + j2 * j2 <= irad2) {
            const float num = __fmul_rn((float)(io[idx] - imin), (float)(USHRT_MAX - 1));
            v = __float2int_rz(__fdiv_rn(num, den));
        }
        io[idx] = v;
        if (out16) out16[idx] = (uint16_t)v;
    }
}

}  // namespace rv

using namespace rv;

extern "C" int RvRescaleSlices(int* d_slices, int nslices, int ixdimp, double center_user, int ipintp,
                               int ibinning, unsigned short* d_out16, int* minmax, void* stream) {
    if (!d_slices || nslices < 1 || ixdimp < 1 || ipintp < 1 || ibinning < 1) {
        set_error(RV_ERR_BAD_ARGUMENT, "RvRescaleSlices: invalid argument");
        return RV_ERR_BAD_ARGUMENT;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // mask radius (source/gazoDoc.cpp:4007-4009), in double as the reference
    const double a = ipintp * center_user / ibinning;
    const double b = ixdimp - ipintp * center_user / ibinning;
    int irad2 = (a < b) ? (int)a : (int)b;
    irad2 *= irad2;
    int* d_mm = nullptr;
    if (!cuda_ok(cudaMallocAsync((void**)&d_mm, sizeof(int) * 2 * nslices, s), RV_ERR_DEVICE_OOM, "min/max"))
        return RV_ERR_DEVICE_OOM;
    std::vector<int> init(2 * nslices);
    for (int k = 0; k < nslices; k++) {
        init[2 * k] = INT_MAX;
        init[2 * k + 1] = 0;
    }
    int rc = 0;
    if (!cuda_ok(cudaMemcpyAsync(d_mm, init.data(), sizeof(int) * 2 * nslices, cudaMemcpyHostToDevice, s),
                 RV_ERR_COPY_H2D, "min/max init"))
        rc = RV_ERR_COPY_H2D;
    if (!rc) {
        const long long n = (long long)ixdimp * ixdimp;
        dim3 g1((unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024), nslices);
        k_minmax<<<g1, 256, 0, s>>>(d_slices, n, d_mm);
        dim3 g2((ixdimp + 255) / 256, ixdimp, nslices);
        k_rescale<<<g2, 256, 0, s>>>(d_slices, d_out16, ixdimp, irad2, d_mm);
        if (!cuda_ok(cudaGetLastError(), RV_ERR_LAUNCH, "rescale kernels")) rc = RV_ERR_LAUNCH;
    }
    if (!rc && minmax) {
        if (!cuda_ok(cudaMemcpyAsync(minmax, d_mm, sizeof(int) * 2 * nslices, cudaMemcpyDeviceToHost, s),
                     RV_ERR_COPY_D2H, "min/max"))
            rc = RV_ERR_COPY_D2H;
    }
    cudaFreeAsync(d_mm, s);
    if (!rc && !cuda_ok(cudaStreamSynchronize(s), RV_ERR_LAUNCH, "rescale")) rc = RV_ERR_LAUNCH;
    return rc;
}
