// selftest.cu — device-side checks of the random stream (host memory in, host memory out).
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include "../../include/arbo.h"
#include "philox.cuh"

namespace {

__global__ void k_philox(const uint32_t* ck, uint32_t n, uint32_t* out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* r = ck + 6 * (size_t)i;
    const arbo::U4 v = arbo::philox4x32_10(r[0], r[1], r[2], r[3], r[4], r[5]);
    for (int k = 0; k < 4; ++k) out[4 * (size_t)i + k] = v.v[k];
}

__global__ void k_curand_philox(unsigned long long seed, uint32_t n, uint32_t* out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    curandStatePhilox4_32_10_t st;
    curand_init(seed, 0, 0, &st);
    for (uint32_t i = 0; i < n; ++i) {
        const uint4 v = curand4(&st);
        out[4 * (size_t)i + 0] = v.x;
        out[4 * (size_t)i + 1] = v.y;
        out[4 * (size_t)i + 2] = v.z;
        out[4 * (size_t)i + 3] = v.w;
    }
}

int run(const void* in, size_t in_bytes, uint32_t* out, size_t out_bytes, int which, unsigned long long seed, uint32_t n)
{
    void* din = nullptr;
    uint32_t* dout = nullptr;
    cudaError_t e = cudaSuccess;
    if (in_bytes && (e = cudaMalloc(&din, in_bytes)) != cudaSuccess) return ARBO_ERR_CUDA;
    if ((e = cudaMalloc(&dout, out_bytes)) != cudaSuccess) {
        cudaFree(din);
        return ARBO_ERR_CUDA;
    }
    if (in_bytes) e = cudaMemcpy(din, in, in_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        if (which == 0) k_philox<<<(n + 255) / 256, 256>>>((const uint32_t*)din, n, dout);
        else k_curand_philox<<<1, 1>>>(seed, n, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, out_bytes, cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(dout);
    return e == cudaSuccess ? ARBO_OK : ARBO_ERR_CUDA;
}

}  // namespace

extern "C" int arbo_selftest_philox(const uint32_t* ctr_key, uint32_t n, uint32_t* out)
{
    if (!ctr_key || !out || n == 0) return ARBO_ERR_INVALID;
    return run(ctr_key, (size_t)n * 6 * 4, out, (size_t)n * 16, 0, 0, n);
}

extern "C" int arbo_selftest_curand_philox(uint64_t seed, uint32_t n, uint32_t* out)
{
    if (!out || n == 0 || n > (1u << 20)) return ARBO_ERR_INVALID;
    return run(nullptr, 0, out, (size_t)n * 16, 1, seed, n);
}
