/*
 * peak.cu: FP32 issue-rate measurement of the device (the denominator of the
 * tracer's roofline).  No counterpart in the reference.
 *
 * Every thread runs 8 independent dependency chains, unrolled, of either
 * plain FP32 additions (one operation a lane and instruction: the rate the
 * bit-exact tracer can reach, since it issues no fused multiply-add) or
 * fused multiply-adds (two operations a lane and instruction).  The grid
 * fills every SM with as many blocks as are resident; the kernel is timed
 * with CUDA events after a warm-up launch, at whatever clock the device
 * runs (no clock is set or locked).
 */
#include <cuda_runtime.h>

#include "qr_gpu.h"

#define QR_PEAK_UNROLL  32
#define QR_PEAK_CHAINS  8

template <int FMA>
__global__ void __launch_bounds__(256)
fp32_issue_kernel(float *out, int iters, float a, float b)
{
    float x[QR_PEAK_CHAINS];
    #pragma unroll
    for (int k = 0; k < QR_PEAK_CHAINS; k++) x[k] = (float)threadIdx.x * 1e-7f + (float)k;
    #pragma unroll 1
    for (int i = 0; i < iters; i++)
    {
        #pragma unroll
        for (int u = 0; u < QR_PEAK_UNROLL; u++)
        {
            #pragma unroll
            for (int k = 0; k < QR_PEAK_CHAINS; k++)
                x[k] = FMA ? __fmaf_rn(x[k], a, b) : __fadd_rn(x[k], b);
        }
    }
    float s = 0.0f;
    #pragma unroll
    for (int k = 0; k < QR_PEAK_CHAINS; k++) s = s + x[k];
    /* keeps the chains live; never true for the arguments passed below */
    if (s == -1.0f) out[blockIdx.x] = s;
}

extern "C" int qr_fp32_peak(int device, int fma, double *tflops)
{
    if (tflops == NULL) return QR_ERR_ARG;
    *tflops = 0.0;
    int prev = -1;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
    if (e != cudaSuccess) return QR_ERR_CUDA;
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess)
        e = fma ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp32_issue_kernel<1>, 256, 0)
                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp32_issue_kernel<0>, 256, 0);
    float *out = NULL;
    cudaEvent_t e0 = NULL, e1 = NULL;
    int rc = QR_OK;
    const int blocks = sms * (per_sm > 0 ? per_sm : 1);
    const int iters = 256;          /* about 0.5 s a launch on a GB300 */
    if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(float) * (size_t)blocks);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.0f;
    for (int rep = 0; rep < 2 && e == cudaSuccess; rep++)
    {
        /* launch 0 warms up, launch 1 is timed */
        e = cudaEventRecord(e0, 0);
        if (fma) fp32_issue_kernel<1><<<blocks, 256>>>(out, iters, 0.999999f, 1e-6f);
        else     fp32_issue_kernel<0><<<blocks, 256>>>(out, iters, 0.999999f, 1e-6f);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e != cudaSuccess) rc = QR_ERR_CUDA;
    else
    {
        const double ops = (double)blocks * 256.0 * iters * QR_PEAK_UNROLL * QR_PEAK_CHAINS *
                           (fma ? 2.0 : 1.0);
        *tflops = ms > 0.0f ? ops / (ms * 1e-3) / 1e12 : 0.0;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    return rc;
}
