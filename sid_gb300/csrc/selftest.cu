// selftest.cu -- self-test of the bounded-wait abort path shared by the
// TMA / tcgen05 kernels (ptx.cuh mbar_wait, gemm_tc.cu's abort handling).
//
// k_selftest_wait has the structure of a pipelined tensor-core kernel at its
// abort point: warp 0 holds a TMEM allocation, thread 0 initialises an
// mbarrier, and warp 1 waits on it.  Nothing is copied and no MMA is issued.
// With `arrive` = 0 nobody arrives, so the bounded wait runs out after `polls`
// polls: the waiter records the timeout code in the error word and raises the
// CTA's abort flag, every warp leaves its role, warp 0 frees TMEM and the
// kernel returns.  The host turns the error word into SID_ETIMEOUT exactly as
// sid_ctx_sync / sid_plan_sync do, and the context stays usable.
#include "ptx.cuh"
#include "sid_internal.cuh"

namespace sid {

__global__ void __launch_bounds__(64, 1) k_selftest_wait(uint32_t polls, int arrive, int* __restrict__ err)
{
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        abort_flag = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "n"(32)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    if (warp == 0 && lane == 0 && arrive) mbar_arrive(&bar);
    if (warp == 1 && lane == 0) {
        if (!mbar_wait_n(&bar, 0, err, polls)) atomicExch(&abort_flag, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(32) : "memory");
    if (threadIdx.x == 0 && abort_flag) atomicExch(err, kErrTimeoutMbar);
}

}  // namespace sid

using namespace sid;

extern "C" int sid_selftest_wait_timeout(uint32_t polls, int arrive)
{
    SID_REQUIRE(polls >= 1 && polls <= (1u << 20), "sid_selftest_wait_timeout: polls must be in [1, 2^20]");
    int* err = nullptr;
    SID_CUDA_TRY(cudaMalloc(&err, sizeof(int)));
    int rc = SID_OK;
    cudaError_t e = cudaMemset(err, 0, sizeof(int));
    if (e == cudaSuccess) {
        k_selftest_wait<<<1, 64>>>(polls, arrive ? 1 : 0, err);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&flag, err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error("sid_selftest_wait_timeout: %s", cudaGetErrorString(e));
        rc = SID_ECUDA;
    } else if (flag) {
        set_error("a device-side wait exceeded its budget (code %d)", flag);
        rc = SID_ETIMEOUT;
    }
    cudaFree(err);
    return rc;
}
