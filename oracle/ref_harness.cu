/* Device helpers of the reference-kernel harness (test infrastructure only; oracle/ref_kernels.py
 * drives them next to the reference's own kernels). Not part of the product library.
 *
 * probe_ids: the reference indexes its curand state array by %smid, %warpid and %laneid
 *   (cpp/cudaidentities.h:14-36, e.g. cpp/ndemographic.cu:88-89), and SM identifiers are not
 *   guaranteed to be contiguous. The harness sizes that array from %nsmid x %nwarpid x 32 and
 *   checks, with a grid that fills every SM, that the identifiers seen stay below both bounds.
 * segment_sums: block b writes the sum of src[b*len .. b*len+len) to dst[b]; used for the daily
 *   incidence per serotype (the reference's d_nIncidenceSubPop is strain-major,
 *   cpp/ndemographic.cu:73) and the live mosquito count.
 */
#include <cstdint>

extern "C" __global__ void probe_ids(uint32_t* out)
{
    uint32_t smid, warpid, nsmid, nwarpid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(warpid));
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(nsmid));
    asm volatile("mov.u32 %0, %%nwarpid;" : "=r"(nwarpid));
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out[0] = nsmid;
        out[1] = nwarpid;
    }
    atomicMax(&out[2], smid);
    atomicMax(&out[3], warpid);
}

extern "C" __global__ void segment_sums(const uint32_t* src, uint32_t* dst, uint32_t len)
{
    __shared__ uint32_t part[32];
    const uint32_t* s = src + (size_t)blockIdx.x * len;
    uint32_t acc = 0;
    for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) acc += s[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) dst[blockIdx.x] = acc;
    }
}
