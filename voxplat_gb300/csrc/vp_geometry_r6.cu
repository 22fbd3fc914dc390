/* vp_geometry_r6.cu — the shell and geometry kernels for chunks of 64^3
 * (k_shell<6>, k_geometry<6>) and their host launchers; the self-test of
 * the decoded-chunk handoff's bounded wait. */
#include "voxgpu.h"
#include "vp_geometry_dev.cuh"

namespace vp {

cudaError_t launch_geometry_r6(const GeoLaunch &L, cudaStream_t st) { return launch_rb<6>(L, st); }
int geometry_ctas_per_sm_r6(int threads) { return ctas_per_sm<6>(threads); }

/* The handoff's bounded wait on a barrier armed for bytes that never come:
 * the wait gives up and the outcome is recorded (vp_selftest_handoff_wait). */
__global__ void k_handoff_wait_selftest(uint32_t *out)
{
	__shared__ __align__(8) uint64_t bar;
	__shared__ uint32_t flag;
	if (threadIdx.x == 0) {
		asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&bar)) : "memory");
		asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
		flag = 0u;
	}
	__syncthreads();
	if (threadIdx.x == 0)
		asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(&bar)), "r"(16u)
			     : "memory");
	if (!mbar_wait(&bar, 0u)) atomicOr(&flag, 1u);
	__syncthreads();
	if (threadIdx.x == 0) *out = flag ? (uint32_t)kStatusTimeout : 0u;
}

} // namespace vp

extern "C" VP_API int vp_selftest_handoff_wait(int device, uint32_t *status)
{
	if (!status) return VP_EINVAL;
	if (cudaSetDevice(device) != cudaSuccess) return VP_ECUDA;
	uint32_t *d = nullptr;
	if (cudaMalloc(&d, sizeof(uint32_t)) != cudaSuccess) return VP_ECUDA;
	vp::k_handoff_wait_selftest<<<1, 32>>>(d);
	cudaError_t e = cudaGetLastError();
	if (e == cudaSuccess) e = cudaMemcpy(status, d, sizeof(uint32_t), cudaMemcpyDeviceToHost);
	cudaFree(d);
	return e == cudaSuccess ? VP_OK : VP_ECUDA;
}
