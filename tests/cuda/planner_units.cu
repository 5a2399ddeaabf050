// Test harness: runs the planner's device pieces (prrtc_gb300/csrc/
// planner_device.cuh) on their own, so that the tests can compare each with
// the oracle's restatement of the reference lines it implements:
//   Halton sampling     halton_next + scale_sample   pRRTC.cu:81-105, Robots.hh
//   nearest neighbour   warp_nn, block_nn            pRRTC.cu:384-412,478-505
//   dynamic domain      dd_grow, dd_shrink           pRRTC.cu:456-468,584-598
// and so that the Halton bases come from the library's own cuRAND shuffle
// (launch_halton_bases).  Built by the tests with nvcc and linked against
// the library; every entry point takes device pointers and synchronises.
#include <cuda_runtime.h>

#include "planner_device.cuh"

namespace prrtc {
cudaError_t launch_halton_bases(float *out, int lanes, cudaStream_t st);
}

using namespace prrtc;

namespace {

template <int D>
__global__ void k_halton(const float *bases16, int lanes, int steps, const float *scale, const float *offset,
                         float *raw, float *cfg)
{
    const int lane = blockIdx.x * blockDim.x + threadIdx.x;
    if (lane >= lanes) return;
    float b[D], n[D], d[D], q[D], sc[D], of[D];
    for (int i = 0; i < D; i++) {
        b[i] = bases16[16 * lane + i];
        n[i] = 0.0f;
        d[i] = 1.0f;
        sc[i] = scale[i];
        of[i] = offset[i];
    }
    for (int s = 0; s < steps; s++) {
        halton_next<D>(b, n, d, q);
        const size_t o = ((size_t)lane * steps + s) * D;
        for (int i = 0; i < D; i++) raw[o + i] = q[i];
        scale_sample<D>(q, sc, of);
        for (int i = 0; i < D; i++) cfg[o + i] = q[i];
    }
}

// one warp per query
template <int D>
__global__ void k_warp_nn(const float *nodes, int cap, int count, const float *q, int nq, int *out_i, float *out_d)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= nq) return;            // whole warps leave together (blockDim a multiple of 32)
    float qq[D];
    for (int i = 0; i < D; i++) qq[i] = q[(size_t)w * D + i];
    float bd;
    int bi;
    warp_nn<D>(nodes, cap, count, qq, bd, bi);
    if (lane_id() == 0) {
        out_i[w] = bi;
        out_d[w] = bd;
    }
}

// one block per query (blockDim <= 256, a multiple of 32)
template <int D>
__global__ void k_block_nn(const float *nodes, int cap, int count, const float *q, int *out_i, float *out_d)
{
    __shared__ float s_q[D], s_red_d[8], s_d;
    __shared__ int s_red_i[8], s_i;
    if (threadIdx.x < D) s_q[threadIdx.x] = q[(size_t)blockIdx.x * D + threadIdx.x];
    __syncthreads();
    block_nn<D>(nodes, cap, count, s_q, s_red_d, s_red_i, &s_d, &s_i);
    if (threadIdx.x == 0) {
        out_i[blockIdx.x] = s_i;
        out_d[blockIdx.x] = s_d;
    }
}

// thread i applies ops[i][0..nops) to radii[i] in order (0 grow, 1 shrink)
__global__ void k_dd_seq(float *radii, int n, const unsigned char *ops, int nops, float alpha, float r0, float rmin)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < nops; k++) {
        if (ops[(size_t)i * nops + k])
            dd_shrink(radii + i, alpha, r0, rmin);
        else
            dd_grow(radii + i, alpha);
    }
}

// every thread of the grid applies op once to the same radius
__global__ void k_dd_contend(float *radius, int op, float alpha, float r0, float rmin)
{
    if (op)
        dd_shrink(radius, alpha, r0, rmin);
    else
        dd_grow(radius, alpha);
}

template <int D>
int nn_run(const float *nodes, int cap, int count, const float *q, int nq, int block, int *oi_w, float *od_w,
           int *oi_b, float *od_b)
{
    if (nq > 0) {
        k_warp_nn<D><<<(nq * 32 + 127) / 128, 128>>>(nodes, cap, count, q, nq, oi_w, od_w);
        k_block_nn<D><<<nq, block>>>(nodes, cap, count, q, oi_b, od_b);
    }
    const cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? (int)cudaGetLastError() : (int)e;
}

template <int D>
int halton_run(const float *bases16, int lanes, int steps, const float *scale, const float *offset, float *raw,
               float *cfg)
{
    if (lanes > 0) k_halton<D><<<(lanes + 63) / 64, 64>>>(bases16, lanes, steps, scale, offset, raw, cfg);
    const cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? (int)cudaGetLastError() : (int)e;
}

}  // namespace

extern "C" {

int units_halton_bases(float *out, int lanes)
{
    cudaError_t e = launch_halton_bases(out, lanes, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return (int)e;
}

int units_halton(int dof, const float *bases16, int lanes, int steps, const float *scale, const float *offset,
                 float *raw, float *cfg)
{
    switch (dof) {
    case 3: return halton_run<3>(bases16, lanes, steps, scale, offset, raw, cfg);
    case 7: return halton_run<7>(bases16, lanes, steps, scale, offset, raw, cfg);
    case 8: return halton_run<8>(bases16, lanes, steps, scale, offset, raw, cfg);
    case 14: return halton_run<14>(bases16, lanes, steps, scale, offset, raw, cfg);
    default: return -1;
    }
}

// nodes: SoA [dof][cap], cap a multiple of 4; q [nq][dof]
int units_nearest(int dof, const float *nodes, int cap, int count, const float *q, int nq, int block, int *oi_w,
                  float *od_w, int *oi_b, float *od_b)
{
    if (cap % 4 || count > cap || block < 32 || block > 256 || block % 32) return -1;
    switch (dof) {
    case 3: return nn_run<3>(nodes, cap, count, q, nq, block, oi_w, od_w, oi_b, od_b);
    case 7: return nn_run<7>(nodes, cap, count, q, nq, block, oi_w, od_w, oi_b, od_b);
    case 8: return nn_run<8>(nodes, cap, count, q, nq, block, oi_w, od_w, oi_b, od_b);
    case 14: return nn_run<14>(nodes, cap, count, q, nq, block, oi_w, od_w, oi_b, od_b);
    default: return -1;
    }
}

int units_dd_seq(float *radii, int n, const unsigned char *ops, int nops, float alpha, float r0, float rmin)
{
    if (n > 0) k_dd_seq<<<(n + 127) / 128, 128>>>(radii, n, ops, nops, alpha, r0, rmin);
    const cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? (int)cudaGetLastError() : (int)e;
}

int units_dd_contend(float *radius, int threads, int op, float alpha, float r0, float rmin)
{
    if (threads >= 128 && threads % 128) return -1;
    if (threads > 0) k_dd_contend<<<(threads + 127) / 128, threads < 128 ? threads : 128>>>(radius, op, alpha, r0, rmin);
    const cudaError_t e = cudaDeviceSynchronize();
    return e == cudaSuccess ? (int)cudaGetLastError() : (int)e;
}

}  // extern "C"
