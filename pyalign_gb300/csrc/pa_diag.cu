// Measured int32 ALU peak of this GPU for the operation mix of the DP cell update
// (add, add, max), used as the roofline denominator of the DP kernels.
#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/pyalign_gb300.h"

namespace {

constexpr int CHAINS = 8;

__global__ void __launch_bounds__(256) int_peak_kernel(int iters, int c1, int c2, int *out) {
	int x[CHAINS], y[CHAINS];
#pragma unroll
	for (int k = 0; k < CHAINS; k++) {
		x[k] = threadIdx.x + k;
		y[k] = blockIdx.x - k;
	}
	for (int i = 0; i < iters; i++) {
#pragma unroll
		for (int k = 0; k < CHAINS; k++) {
			const int t = max(x[k] + c1, y[k] + c2);  // 3 int ops
			y[k] = x[k];
			x[k] = t;
		}
	}
	int s = 0;
#pragma unroll
	for (int k = 0; k < CHAINS; k++) s ^= x[k] + y[k];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" pa_status pa_measure_int32_peak(float *gops, float *ms_out) {
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return PA_ERR_NO_DEVICE;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const int blocks = sms * 8, threads = 256, iters = 1 << 14;
	int *out = nullptr;
	if (cudaMalloc(&out, size_t(blocks) * threads * sizeof(int)) != cudaSuccess) return PA_ERR_CUDA;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	int_peak_kernel<<<blocks, threads>>>(iters, 3, -5, out);  // warm-up
	float best = 1e30f;
	for (int rep = 0; rep < 5; rep++) {
		cudaEventRecord(e0);
		int_peak_kernel<<<blocks, threads>>>(iters, 3, -5, out);
		cudaEventRecord(e1);
		cudaEventSynchronize(e1);
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (ms < best) best = ms;
	}
	const cudaError_t err = cudaGetLastError();
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	cudaFree(out);
	if (err != cudaSuccess) return PA_ERR_CUDA;
	const double ops = double(blocks) * threads * iters * CHAINS * 3.0;
	if (gops) *gops = float(ops / (best * 1e-3) / 1e9);
	if (ms_out) *ms_out = best;
	return PA_OK;
}
