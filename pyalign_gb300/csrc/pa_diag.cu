// Measured ALU peaks of this GPU for the operation mix of the DP cell update (add, add,
// max): on int32 lanes, the roofline denominator of the int32 DP kernels; on packed 16-bit
// pairs, that of the 16-bit twin kernel; on float32, that of the float DP kernels.
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

// The same mix on packed 16-bit pairs (add.s16x2, max.s16x2): each instruction does two
// lane operations.
__global__ void __launch_bounds__(256) int16x2_peak_kernel(int iters, uint32_t c1, uint32_t c2, uint32_t *out) {
	uint32_t x[CHAINS], y[CHAINS];
#pragma unroll
	for (int k = 0; k < CHAINS; k++) {
		x[k] = threadIdx.x * 0x10001u + k;
		y[k] = blockIdx.x * 0x10001u - k;
	}
	for (int i = 0; i < iters; i++) {
#pragma unroll
		for (int k = 0; k < CHAINS; k++) {
			uint32_t a, b, t;
			asm("add.s16x2 %0, %1, %2;" : "=r"(a) : "r"(x[k]), "r"(c1));
			asm("add.s16x2 %0, %1, %2;" : "=r"(b) : "r"(y[k]), "r"(c2));
			asm("max.s16x2 %0, %1, %2;" : "=r"(t) : "r"(a), "r"(b));  // 3 packed ops
			y[k] = x[k];
			x[k] = t;
		}
	}
	uint32_t s = 0;
#pragma unroll
	for (int k = 0; k < CHAINS; k++) s ^= x[k] + y[k];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The same mix in float32 (two adds, one max per chain step), the arithmetic of the float
// DP kernels (similarity-matrix and DTW forms).
__global__ void __launch_bounds__(256) f32_peak_kernel(int iters, float c1, float c2, float *out) {
	float x[CHAINS], y[CHAINS];
#pragma unroll
	for (int k = 0; k < CHAINS; k++) {
		x[k] = float(threadIdx.x + k);
		y[k] = float(blockIdx.x) - float(k);
	}
	for (int i = 0; i < iters; i++) {
#pragma unroll
		for (int k = 0; k < CHAINS; k++) {
			const float t = fmaxf(x[k] + c1, y[k] + c2);  // 3 float ops
			y[k] = x[k];
			x[k] = t;
		}
	}
	float s = 0.0f;
#pragma unroll
	for (int k = 0; k < CHAINS; k++) s += x[k] - y[k];
	out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename K, typename C>
pa_status time_peak(K kernel, C c1, C c2, double ops_per_chain_step, float *gops, float *ms_out) {
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return PA_ERR_NO_DEVICE;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	const int blocks = sms * 8, threads = 256, iters = 1 << 14;
	C *out = nullptr;
	if (cudaMalloc(&out, size_t(blocks) * threads * sizeof(C)) != cudaSuccess) return PA_ERR_CUDA;
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	kernel<<<blocks, threads>>>(iters, c1, c2, out);  // warm-up
	float best = 1e30f;
	for (int rep = 0; rep < 5; rep++) {
		cudaEventRecord(e0);
		kernel<<<blocks, threads>>>(iters, c1, c2, out);
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
	const double ops = double(blocks) * threads * iters * CHAINS * ops_per_chain_step;
	if (gops) *gops = float(ops / (best * 1e-3) / 1e9);
	if (ms_out) *ms_out = best;
	return PA_OK;
}

}  // namespace

extern "C" pa_status pa_measure_int16x2_peak(float *gops, float *ms_out) {
	return time_peak(int16x2_peak_kernel, 0x00030003u, 0xFFFBFFFBu, 6.0, gops, ms_out);
}

extern "C" pa_status pa_measure_f32_peak(float *gops, float *ms_out) {
	return time_peak(f32_peak_kernel, 0.5f, -0.25f, 3.0, gops, ms_out);
}

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
