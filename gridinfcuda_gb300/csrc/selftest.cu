// selftest.cu -- exercises the bounded device-side waits (ptx.cuh) on
// purpose: an mbarrier phase nothing completes and a grid barrier one block
// short.  Each wait gives up after its time limit, records DEV_ERR_TIMEOUT in
// the status word and returns, so the kernels end normally and the context
// stays usable; the host reads the status words.  No fault, trap or unbounded
// loop is involved.
#include "ginf_gb300.h"
#include "ginf_internal.h"
#include "ptx.cuh"

namespace ginf_gpu {
namespace {

// One thread waits on an mbarrier that expects one arrival which never comes.
__global__ void k_wait_mbarrier(int *status) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait_bounded(&bar, 0, status);
}

// Every block meets at a grid barrier told to expect one block more than
// the launch has.
__global__ void k_wait_grid_barrier(unsigned int *bar, unsigned int expected, int *status) {
    grid_barrier(bar, expected, status);
}

}  // namespace
}  // namespace ginf_gpu

using namespace ginf_gpu;

extern "C" ginf_status ginf_selftest_bounded_waits(int32_t *mbarrier_status, int32_t *barrier_status) {
    set_last_error("");
    if (!mbarrier_status || !barrier_status) {
        set_last_error("NULL argument");
        return GINF_ERR_INVALID_ARGUMENT;
    }
    int *dev = nullptr;
    cudaError_t e = cudaMalloc(&dev, 64);
    if (e == cudaSuccess) e = cudaMemset(dev, 0, 64);
    if (e == cudaSuccess) {
        k_wait_mbarrier<<<1, 32>>>(dev);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        // Two co-resident blocks (a cooperative launch) wait for a third.
        unsigned int *bar = reinterpret_cast<unsigned int *>(dev + 8);
        unsigned int expected = 3;
        int *st = dev + 1;
        void *args[] = {&bar, &expected, &st};
        e = cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k_wait_grid_barrier), dim3(2), dim3(32), args,
                                        0, nullptr);
    }
    int host[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(host, dev, sizeof(host), cudaMemcpyDeviceToHost);
    if (dev) cudaFree(dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error(cudaGetErrorString(e));
        return GINF_ERR_CUDA;
    }
    *mbarrier_status = host[0];
    *barrier_status = host[1];
    return GINF_OK;
}
