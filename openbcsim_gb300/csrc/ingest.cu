// ingest.cu -- device-side ingestion of scatterer datasets.
//
// add_fixed_scatterers / add_spline_scatterers copy the caller's arrays to the
// device as they are and finish there: the spline control points are laid out
// [K][N] float4 for the kernels (the caller's layout is [N][K][3], pyrfsim's,
// PythonInterface.cpp:140-160), and the amplitude bound of the fixed-point scale
// (sum of |a|) and the non-finite check (CpuAlgorithm.cpp:81-83 under
// BCSIM_ENABLE_NAN_CHECK) are reductions -- done in a fixed order, so the same
// data always gives the same bound.
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>
#include "kernels.hpp"

namespace bcsim_gb300 {

constexpr int SUM_THREADS = 256;
constexpr int SUM_BLOCKS = 512;

// out[k * n + i] = (raw[i][k][0..2], 0)
__global__ void spline_transpose_kernel(const float* __restrict__ raw, int64_t n, int K, float4* __restrict__ out) {
    const int64_t total = n * (int64_t)K;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / n, i = t - k * n;
        const float* q = raw + (i * K + k) * 3;
        out[t] = make_float4(__ldg(q), __ldg(q + 1), __ldg(q + 2), 0.0f);
    }
}

// Per-block partial sums of |vals[i * stride]| in double: thread j adds
// elements j, j + G, j + 2G, ... (G = the grid's threads), then a fixed
// shared-memory tree; non-finite values are counted apart.
__global__ void __launch_bounds__(SUM_THREADS)
    abs_sum_partial_kernel(const float* __restrict__ vals, int64_t stride, int64_t n, double* __restrict__ partial,
                           int* __restrict__ nonfinite) {
    __shared__ double sh[SUM_THREADS];
    double s = 0.0;
    int bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * SUM_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * SUM_THREADS) {
        const float a = __ldg(vals + i * stride);
        if (isfinite(a)) s += fabs((double)a);
        else bad = 1;
    }
    sh[threadIdx.x] = s;
    if (bad) atomicOr(nonfinite, 1);
    __syncthreads();
    for (int w = SUM_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(SUM_THREADS) abs_sum_final_kernel(const double* __restrict__ partial, int blocks,
                                                                   double* __restrict__ out) {
    __shared__ double sh[SUM_THREADS];
    double s = 0.0;
    for (int b = threadIdx.x; b < blocks; b += SUM_THREADS) s += partial[b];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = SUM_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = sh[0];
}

cudaError_t launch_spline_transpose(const float* raw, int64_t n, int num_cs, float4* out, cudaStream_t stream) {
    const int64_t total = n * (int64_t)num_cs;
    if (total <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 32);
    spline_transpose_kernel<<<(unsigned)blocks, 256, 0, stream>>>(raw, n, num_cs, out);
    return cudaGetLastError();
}

size_t abs_sum_scratch_bytes() { return (SUM_BLOCKS + 1) * sizeof(double) + sizeof(int); }

cudaError_t abs_sum_enqueue(const float* vals, int64_t stride, int64_t n, void* scratch, double* sum, int* nonfinite,
                            cudaStream_t stream) {
    double* partial = static_cast<double*>(scratch);
    double* out = partial + SUM_BLOCKS;
    int* bad = reinterpret_cast<int*>(out + 1);
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) + sizeof(int), stream);
    if (e != cudaSuccess) return e;
    if (n > 0) {
        abs_sum_partial_kernel<<<SUM_BLOCKS, SUM_THREADS, 0, stream>>>(vals, stride, n, partial, bad);
        abs_sum_final_kernel<<<1, SUM_THREADS, 0, stream>>>(partial, SUM_BLOCKS, out);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = cudaMemcpyAsync(sum, out, sizeof(double), cudaMemcpyDeviceToHost, stream)) != cudaSuccess) return e;
    return cudaMemcpyAsync(nonfinite, bad, sizeof(int), cudaMemcpyDeviceToHost, stream);
}

cudaError_t abs_sum(const float* vals, int64_t stride, int64_t n, void* scratch, double* sum, int* nonfinite,
                    cudaStream_t stream) {
    *sum = 0.0;
    *nonfinite = 0;
    if (n <= 0) return cudaSuccess;
    cudaError_t e = abs_sum_enqueue(vals, stride, n, scratch, sum, nonfinite, stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(stream);
}

}  // namespace bcsim_gb300
