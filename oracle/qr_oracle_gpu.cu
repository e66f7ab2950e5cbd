/*
 * qr_oracle_gpu.cu: the FP64 path-tracer oracle on the GPU.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the path tracer's means at sizes
 * and sample counts the host restatement cannot reach in a test's time
 * (the 1280x720 path-traced frame at 4096 samples a pixel).  Nothing in the
 * product links this file.
 *
 * It compiles the restatement qr_oracle.c in double precision
 * (QR_ORACLE_FP64) for the device: threads run the oracle's per-pixel
 * estimator over slices of a pixel's samples (pt_pixel: the reference's
 * path-tracer sample loop,
 * core/tracer/tracer.cpp 2115-2139, 3428-3666, 4685-4723, with the same
 * counter-based draws as the float tracer) over rows [y0, y1) of a frame.
 * Each sample's arithmetic is the host FP64 oracle's, instruction for
 * instruction (the device's double-precision + - * / sqrt fma all round to
 * nearest as the host's do); only the order in which a pixel's sample values
 * are summed differs (slices of ORACLE_SPT samples, then slice sums).
 */
#define QR_ORACLE_FP64 1
#include "qr_oracle.c"

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <chrono>

/* samples [n_base + s * spt, n_base + (s + 1) * spt) of one band pixel, for
 * slot s of the launch: the draws are counter-based (keyed by the sample
 * number), so a pixel's samples split over threads give the same samples */
__global__ void oracle_pt_part(qr_scene_desc d, qr_frame_params fp, double *part, int y0,
                               int y1, int n_base, int spt, int slots)
{
    const long long npx = (long long)(y1 - y0) * fp.x_res;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npx * slots) return;
    const int s = (int)(t / npx);
    const long long i = t - (long long)s * npx;   /* neighbouring threads: neighbouring pixels */
    const int x = (int)(i % fp.x_res), y = y0 + (int)(i / fp.x_res);
    scene_t sc;
    scene_of(&sc, &d, &fp);
    qr_frame_params q = fp;
    q.pt_on = spt;
    q.pts_c = (float)(n_base + s * spt);
    double a[3] = {0.0, 0.0, 0.0};
    (void)pt_pixel(&sc, &d, &q, x, y, a);
    double *o = part + 3 * (size_t)t;
    o[0] = a[0];
    o[1] = a[1];
    o[2] = a[2];
}

#define ORACLE_SPT   8          /* samples a thread */
#define ORACLE_SLOTS 32         /* threads a pixel in one launch */

/* rows [y0, y1) of the path-traced frame in double precision on the GPU:
 * acc receives the sums (3 doubles a pixel) and frame the packed means, both
 * band-sized with an x_res stride (host memory); fp->pts_c must be 0.
 * The samples run in launches of ORACLE_SPT x ORACLE_SLOTS samples a pixel;
 * each launch's per-thread sums are added on the host, slot after slot, so
 * the result does not depend on timing.  After each launch the call gives up
 * once max_s seconds have passed: it then returns -2 with *done the samples
 * a pixel summed so far.  Returns 0, -1 for bad arguments, -2, or a CUDA
 * error code */
extern "C" int qr_oracle_pt_gpu(const qr_scene_desc *d, const qr_frame_params *fp,
                                double *acc, uint32_t *frame, int y0, int y1, double max_s,
                                int *done)
{
    if (fp->pts_c != 0.0f || y0 < 0 || y1 > fp->y_res || y0 >= y1 || fp->pt_on <= 0 ||
        fp->pt_on % (ORACLE_SPT * ORACLE_SLOTS) != 0)
        return -1;
    const size_t npx = (size_t)(y1 - y0) * fp->x_res;
    const size_t nthr = npx * ORACLE_SLOTS;
    const size_t sz[6] = {sizeof(qr_srf) * d->nsrf, sizeof(qr_mat) * d->nmat,
                          sizeof(qr_light) * d->nlgt, sizeof(qr_elem) * d->nelem,
                          sizeof(qr_lelem) * d->nlelem, sizeof(uint32_t) * d->ntex};
    const void *src[6] = {d->srf, d->mat, d->lgt, d->elems, d->lelems, d->texels};
    void *dst[6] = {NULL, NULL, NULL, NULL, NULL, NULL};
    double *dpart = NULL, *hpart = NULL;
    size_t old_stack = 0;
    int rc = 0;
    if (done) *done = 0;
    for (size_t i = 0; i < npx * 3; i++) acc[i] = 0.0;
    hpart = (double *)malloc(nthr * 3 * sizeof(double));
    if (hpart == NULL) return -1;
    /* the estimator recurses per tree level (up to depth + 1 frames) */
    cudaError_t e = cudaDeviceGetLimit(&old_stack, cudaLimitStackSize);
    if (e == cudaSuccess) e = cudaDeviceSetLimit(cudaLimitStackSize, 16384);
    for (int k = 0; k < 6 && e == cudaSuccess; k++)
    {
        e = cudaMalloc(&dst[k], sz[k] > 0 ? sz[k] : 16);
        if (e == cudaSuccess && sz[k] > 0) e = cudaMemcpy(dst[k], src[k], sz[k], cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&dpart, nthr * 3 * sizeof(double));
    qr_scene_desc dd = *d;
    dd.srf = (const qr_srf *)dst[0];
    dd.mat = (const qr_mat *)dst[1];
    dd.lgt = (const qr_light *)dst[2];
    dd.elems = (const qr_elem *)dst[3];
    dd.lelems = (const qr_lelem *)dst[4];
    dd.texels = (const uint32_t *)dst[5];
    const auto t0 = std::chrono::steady_clock::now();
    const int per_launch = ORACLE_SPT * ORACLE_SLOTS;
    for (int n = 0; n < fp->pt_on && e == cudaSuccess; n += per_launch)
    {
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (n > 0 && el > max_s) { rc = -2; break; }
        const unsigned blocks = (unsigned)((nthr + 127) / 128);
        oracle_pt_part<<<blocks, 128>>>(dd, *fp, dpart, y0, y1, n, ORACLE_SPT, ORACLE_SLOTS);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(hpart, dpart, nthr * 3 * sizeof(double),
                                             cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) break;
        for (int s = 0; s < ORACLE_SLOTS; s++)
            for (size_t i = 0; i < npx * 3; i++) acc[i] += hpart[(size_t)s * npx * 3 + i];
        if (done) *done = n + per_launch;
    }
    if (e == cudaSuccess && rc == 0)
    {
        for (size_t i = 0; i < npx; i++)
        {
            real m[3];
            for (int k = 0; k < 3; k++) m[k] = clamp1(acc[3 * i + k] / (real)fp->pt_on);
            frame[i] = pack(fp, m);
        }
    }
    for (int k = 0; k < 6; k++)
        if (dst[k]) cudaFree(dst[k]);
    if (dpart) cudaFree(dpart);
    free(hpart);
    if (old_stack) cudaDeviceSetLimit(cudaLimitStackSize, old_stack);
    if (e != cudaSuccess) fprintf(stderr, "qr_oracle_pt_gpu: %s\n", cudaGetErrorString(e));
    return e != cudaSuccess ? (int)e : rc;
}
