// Batch encoding of byte-alphabet sequences into the index codes of the indexed form.
//
// Replaces the per-problem encoding of pyalign's prepare step (pyalign/solve.py:382-396
// calls AlphabetProblem.build_index_sequences for every problem of a batch,
// pyalign/problems/factory.py:87-90, which encodes each string with
// ByteAlphabetEncoder.encode, factory.py:103-127: latin1 bytes mapped through a 256-entry
// index table, 0xff = not in the alphabet -> ValueError("item not in alphabet")).  Here one
// call encodes all strings of a batch: on the host by worker threads, or on the device from
// one upload of the raw bytes (a quarter of the uint32 codes' size).
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include <string>
#include "../../include/pyalign_gb300.h"

namespace pa {
pa_status wsb_fail(pa_status st, const std::string &m);  // the library's error slot (pa_last_error)
}  // namespace pa

namespace {

constexpr int ENC_BAD_BYTE = 1;
constexpr int ENC_TOO_LONG = 2;

// One warp per string: lane i maps bytes i, i + 32, ...; the row is zero-padded to width.
__global__ void encode_latin1_kernel(const uint8_t *text, const int64_t *offsets, int64_t count, const uint8_t *lut,
                                     int64_t width, int64_t stride, uint32_t *codes, int32_t *flags) {
	__shared__ uint8_t tab[256];
	for (int k = threadIdx.x; k < 256; k += blockDim.x) tab[k] = lut[k];
	__syncthreads();
	const int lane = threadIdx.x & 31;
	const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
	for (int64_t s = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; s < count; s += warps) {
		const int64_t o0 = offsets[s], n = offsets[s + 1] - o0;
		if (n > width) {
			if (lane == 0) atomicOr(flags, ENC_TOO_LONG);
			continue;
		}
		uint32_t *row = codes + s * stride;
		bool bad = false;
		for (int64_t i = lane; i < width; i += 32) {
			uint32_t c = 0;
			if (i < n) {
				c = tab[text[o0 + i]];
				bad |= c == 0xffu;
			}
			row[i] = c;
		}
		if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(flags, ENC_BAD_BYTE);
	}
}

pa_status encode_error(int flags) {
	if (flags & ENC_TOO_LONG) return pa::wsb_fail(PA_ERR_LENGTH, "sequence longer than the code array's width");
	if (flags & ENC_BAD_BYTE) return pa::wsb_fail(PA_ERR_INVALID_ARGUMENT, "item not in alphabet");  // factory.py:121-122
	return PA_OK;
}

}  // namespace

extern "C" pa_status pa_encode_latin1(const uint8_t *text, const int64_t *offsets, int64_t count, const uint8_t *lut,
                                      int64_t width, int64_t row_stride, uint32_t *codes, int32_t location,
                                      void *stream) {
	if (count < 0 || width < 0 || row_stride < width || !offsets || !lut || (count > 0 && !codes))
		return pa::wsb_fail(PA_ERR_INVALID_ARGUMENT, "pa_encode_latin1: invalid arguments");
	if (count == 0) return PA_OK;
	for (int64_t k = 0; k < count; k++)
		if (offsets[k + 1] < offsets[k]) return pa::wsb_fail(PA_ERR_INVALID_ARGUMENT, "pa_encode_latin1: offsets decrease");
	const int64_t nbytes = offsets[count] - offsets[0];
	if (nbytes > 0 && !text) return pa::wsb_fail(PA_ERR_INVALID_ARGUMENT, "pa_encode_latin1: null text");

	if (location == PA_HOST) {
		// worker threads over contiguous string ranges
		const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
		const int64_t nth = std::max<int64_t>(1, std::min<int64_t>(hw, (nbytes + count * 8) / (1 << 20) + 1));
		std::atomic<int> flags{0};
		auto work = [&](int64_t s0, int64_t s1) {
			int f = 0;
			for (int64_t s = s0; s < s1; s++) {
				const int64_t o0 = offsets[s], n = offsets[s + 1] - o0;
				if (n > width) {
					f |= ENC_TOO_LONG;
					continue;
				}
				uint32_t *row = codes + s * row_stride;
				uint8_t acc = 0;
				for (int64_t i = 0; i < n; i++) {
					const uint8_t c = lut[text[o0 + i]];
					acc |= uint8_t(c == 0xffu);
					row[i] = c;
				}
				if (acc) f |= ENC_BAD_BYTE;
				std::memset(row + n, 0, size_t(width - n) * sizeof(uint32_t));
			}
			if (f) flags.fetch_or(f);
		};
		if (nth == 1) {
			work(0, count);
		} else {
			std::vector<std::thread> pool;
			for (int64_t t = 0; t < nth; t++) pool.emplace_back(work, count * t / nth, count * (t + 1) / nth);
			for (auto &th : pool) th.join();
		}
		return encode_error(flags.load());
	}
	if (location != PA_DEVICE) return pa::wsb_fail(PA_ERR_INVALID_ARGUMENT, "pa_encode_latin1: bad location");

	// device: one upload of the bytes, the offsets and the table, one kernel
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	const size_t off_bytes = size_t(count + 1) * sizeof(int64_t);
	const size_t head = (off_bytes + 256 + sizeof(int32_t) + 15) & ~size_t(15);
	unsigned char *buf = nullptr;
	if (cudaMallocAsync(reinterpret_cast<void **>(&buf), head + size_t(std::max<int64_t>(nbytes, 1)), st) != cudaSuccess)
		return pa::wsb_fail(PA_ERR_CUDA, "pa_encode_latin1: device allocation failed");
	int64_t *d_off = reinterpret_cast<int64_t *>(buf);
	uint8_t *d_lut = buf + off_bytes;
	int32_t *d_flags = reinterpret_cast<int32_t *>(buf + off_bytes + 256);
	uint8_t *d_text = buf + head;
	std::vector<int64_t> rel(static_cast<size_t>(count + 1));
	for (int64_t k = 0; k <= count; k++) rel[size_t(k)] = offsets[k] - offsets[0];
	int32_t flags = 0;
	cudaError_t e = cudaMemcpyAsync(d_off, rel.data(), off_bytes, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(d_lut, lut, 256, cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) e = cudaMemsetAsync(d_flags, 0, sizeof(int32_t), st);
	if (e == cudaSuccess && nbytes > 0) e = cudaMemcpyAsync(d_text, text + offsets[0], size_t(nbytes), cudaMemcpyHostToDevice, st);
	if (e == cudaSuccess) {
		int dev = 0, sms = 1;
		cudaGetDevice(&dev);
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		const int64_t blocks = std::min<int64_t>(int64_t(sms) * 8, (count + 7) / 8);
		encode_latin1_kernel<<<int(std::max<int64_t>(blocks, 1)), 256, 0, st>>>(d_text, d_off, count, d_lut, width,
		                                                                       row_stride, codes, d_flags);
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, d_flags, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
	cudaFreeAsync(buf, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return pa::wsb_fail(PA_ERR_CUDA, std::string("pa_encode_latin1: ") + cudaGetErrorString(e));
	return encode_error(flags);
}
