/*
 * qr_oracle_gpu.cu: the FP64 path-tracer oracle on the GPU.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the path tracer's means at sizes
 * and sample counts the host restatement cannot reach in a test's time
 * (the 1280x720 path-traced frame at 4096 samples a pixel).  Nothing in the
 * product links this file.
 *
 * It compiles the restatement qr_oracle.c in double precision
 * (QR_ORACLE_FP64) for the device: one thread a pixel runs the oracle's
 * per-pixel estimator (pt_pixel: the reference's path-tracer sample loop,
 * core/tracer/tracer.cpp 2115-2139, 3428-3666, 4685-4723, with the same
 * counter-based draws as the float tracer) over rows [y0, y1) of a frame.
 * Its arithmetic is the host FP64 oracle's, instruction for instruction,
 * apart from what the device's double-precision operations round
 * differently (none of + - * / sqrt fma: all are IEEE round-to-nearest).
 */
#define QR_ORACLE_FP64 1
#include "qr_oracle.c"

#include <cuda_runtime.h>
#include <stdio.h>

__global__ void oracle_pt_kernel(qr_scene_desc d, qr_frame_params fp, double *acc,
                                 uint32_t *frame, int y0, int y1)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = y0 + blockIdx.y;
    if (x >= fp.x_res || y >= y1) return;
    scene_t sc;
    scene_of(&sc, &d, &fp);
    const size_t i = (size_t)(y - y0) * fp.x_res + x;
    frame[i] = pt_pixel(&sc, &d, &fp, x, y, acc + 3 * i);
}

/* rows [y0, y1) of the path-traced frame in double precision on the GPU:
 * acc receives the sums (3 doubles a pixel) and frame the packed means, both
 * band-sized with an x_res stride (host memory); fp->pts_c must be 0.
 * Returns 0, or a CUDA error code */
extern "C" int qr_oracle_pt_gpu(const qr_scene_desc *d, const qr_frame_params *fp,
                                double *acc, uint32_t *frame, int y0, int y1)
{
    if (fp->pts_c != 0.0f || y0 < 0 || y1 > fp->y_res || y0 >= y1 || fp->pt_on <= 0)
        return -1;
    const size_t npx = (size_t)(y1 - y0) * fp->x_res;
    const size_t sz[6] = {sizeof(qr_srf) * d->nsrf, sizeof(qr_mat) * d->nmat,
                          sizeof(qr_light) * d->nlgt, sizeof(qr_elem) * d->nelem,
                          sizeof(qr_lelem) * d->nlelem, sizeof(uint32_t) * d->ntex};
    const void *src[6] = {d->srf, d->mat, d->lgt, d->elems, d->lelems, d->texels};
    void *dst[6] = {NULL, NULL, NULL, NULL, NULL, NULL};
    double *dacc = NULL;
    uint32_t *dframe = NULL;
    size_t old_stack = 0;
    /* the estimator recurses per tree level (up to depth + 1 frames) */
    cudaError_t e = cudaDeviceGetLimit(&old_stack, cudaLimitStackSize);
    if (e == cudaSuccess) e = cudaDeviceSetLimit(cudaLimitStackSize, 16384);
    for (int k = 0; k < 6 && e == cudaSuccess; k++)
    {
        e = cudaMalloc(&dst[k], sz[k] > 0 ? sz[k] : 16);
        if (e == cudaSuccess && sz[k] > 0) e = cudaMemcpy(dst[k], src[k], sz[k], cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&dacc, npx * 3 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dframe, npx * sizeof(uint32_t));
    if (e == cudaSuccess)
    {
        qr_scene_desc dd = *d;
        dd.srf = (const qr_srf *)dst[0];
        dd.mat = (const qr_mat *)dst[1];
        dd.lgt = (const qr_light *)dst[2];
        dd.elems = (const qr_elem *)dst[3];
        dd.lelems = (const qr_lelem *)dst[4];
        dd.texels = (const uint32_t *)dst[5];
        const dim3 block(64, 1), grid((fp->x_res + 63) / 64, y1 - y0);
        oracle_pt_kernel<<<grid, block>>>(dd, *fp, dacc, dframe, y0, y1);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) e = cudaMemcpy(acc, dacc, npx * 3 * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(frame, dframe, npx * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    for (int k = 0; k < 6; k++)
        if (dst[k]) cudaFree(dst[k]);
    if (dacc) cudaFree(dacc);
    if (dframe) cudaFree(dframe);
    if (old_stack) cudaDeviceSetLimit(cudaLimitStackSize, old_stack);
    if (e != cudaSuccess) fprintf(stderr, "qr_oracle_pt_gpu: %s\n", cudaGetErrorString(e));
    return (int)e;
}
