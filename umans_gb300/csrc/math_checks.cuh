// device exception tables of the reference-exact sinf/cosf/expf and their
// test entry points
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

// Sets this module's sinf/cosf exception tables on the current device (once).
bool set_device_sincos(std::string& err)
{
	static std::mutex mu;
	static std::set<int> done;
	std::lock_guard<std::mutex> lk(mu);
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) { err = "cudaGetDevice failed"; return false; }
	if (done.count(dev)) return true;
	SinCosExceptions T;
	if (!sincos_exceptions_for_device(&T, nullptr, err)) return false;
	const cudaError_t e = cudaMemcpyToSymbol(c_sincos, &T, sizeof(T));
	if (e != cudaSuccess) { err = std::string("sincos table: ") + cudaGetErrorString(e); return false; }
	done.insert(dev);
	return true;
}

__global__ void k_ref_sincosf(const float* x, float* s, float* c, int n)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) host_sincosf(x[i], &s[i], &c[i]);
}

// Evaluates the device's reference-exact sinf/cosf on n host values (tests).
bool debug_ref_sincosf(const float* x, float* s, float* c, int n, size_t* exceptions, std::string& err)
{
	if (!set_device_sincos(err)) return false;
	if (exceptions) {
		SinCosExceptions T;
		if (!sincos_exceptions_for_device(&T, exceptions, err)) return false;
	}
	float *dx = nullptr, *ds = nullptr, *dc = nullptr;
	const size_t b = sizeof(float) * std::max(n, 1);
	if (cudaMalloc(&dx, b) != cudaSuccess || cudaMalloc(&ds, b) != cudaSuccess || cudaMalloc(&dc, b) != cudaSuccess) {
		err = "cudaMalloc";
		return false;
	}
	cudaMemcpy(dx, x, sizeof(float) * n, cudaMemcpyHostToDevice);
	if (n > 0) k_ref_sincosf<<<(n + 255) / 256, 256>>>(dx, ds, dc, n);
	cudaError_t e = cudaMemcpy(s, ds, sizeof(float) * n, cudaMemcpyDeviceToHost);
	if (e == cudaSuccess) e = cudaMemcpy(c, dc, sizeof(float) * n, cudaMemcpyDeviceToHost);
	cudaFree(dx);
	cudaFree(ds);
	cudaFree(dc);
	if (e != cudaSuccess) { err = cudaGetErrorString(e); return false; }
	return true;
}

__global__ void k_ref_expf(ExpExceptions T, const float* x, float* y, int n)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) y[i] = ref_expf(T, x[i]);
}

// Evaluates the device's reference-exact expf on n host values (tests).
__global__ void k_prod_diff(const float4* abcd, float* y, int n)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) {
		const float4 q = abcd[i];
		y[i] = prod_diff_d(q.x, q.y, q.z, q.w);
	}
}

// Evaluates the device's (float)((double)a*b - (double)c*d) on n host
// quadruples (tests).
bool debug_prod_diff(const float* abcd, float* y, int n, std::string& err)
{
	float4* dq = nullptr;
	float* dy = nullptr;
	if (cudaMalloc(&dq, sizeof(float4) * std::max(n, 1)) != cudaSuccess ||
	    cudaMalloc(&dy, sizeof(float) * std::max(n, 1)) != cudaSuccess) { err = "cudaMalloc"; return false; }
	cudaMemcpy(dq, abcd, sizeof(float4) * n, cudaMemcpyHostToDevice);
	if (n > 0) k_prod_diff<<<(n + 255) / 256, 256>>>(dq, dy, n);
	cudaError_t e = cudaMemcpy(y, dy, sizeof(float) * n, cudaMemcpyDeviceToHost);
	cudaFree(dq);
	cudaFree(dy);
	if (e != cudaSuccess) { err = cudaGetErrorString(e); return false; }
	return true;
}

bool debug_ref_expf(const float* x, float* y, int n, size_t* exceptions, std::string& err)
{
	ExpExceptions T;
	if (!exp_exceptions_for_device(&T, exceptions, err)) return false;
	float *dx = nullptr, *dy = nullptr;
	if (cudaMalloc(&dx, sizeof(float) * std::max(n, 1)) != cudaSuccess ||
	    cudaMalloc(&dy, sizeof(float) * std::max(n, 1)) != cudaSuccess) { err = "cudaMalloc"; return false; }
	cudaMemcpy(dx, x, sizeof(float) * n, cudaMemcpyHostToDevice);
	if (n > 0) k_ref_expf<<<(n + 255) / 256, 256>>>(T, dx, dy, n);
	cudaError_t e = cudaMemcpy(y, dy, sizeof(float) * n, cudaMemcpyDeviceToHost);
	cudaFree(dx);
	cudaFree(dy);
	if (e != cudaSuccess) { err = cudaGetErrorString(e); return false; }
	return true;
}

// The short exponential against the table-backed one on the float bit
// patterns [first, first + count) that lie in [-87, 0].  counts[0]: values
// where it answered, [1]: of those, results that differ from ff_expf_core,
// [2]: answered values that the exception table lists.
__global__ void k_expf_check(ExpExceptions T, uint32_t first, uint32_t count, unsigned long long* counts)
{
	unsigned long long dec = 0, bad = 0, listed = 0;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
		const uint32_t b = first + i;
		const float x = __uint_as_float(b);
		if (!(x >= FF_EXP_LO && x <= 0.0f)) continue;
		float y;
		if (!exp_fast(x, T.band, &y)) continue;
		++dec;
		const float z = ff_expf_core(x);
		bool in_table = false;
		uint32_t h = ff_hash(b, T.shift);
		for (;;) {
			const uint2 e = T.slots[h];
			if (e.x == 0) break;
			if (e.x == b) { in_table = true; break; }
			h = (h + 1) & T.mask;
		}
		listed += in_table;
		bad += __float_as_uint(y) != __float_as_uint(z);
	}
	for (int o = 16; o > 0; o >>= 1) {
		dec += __shfl_xor_sync(0xffffffffu, dec, o);
		bad += __shfl_xor_sync(0xffffffffu, bad, o);
		listed += __shfl_xor_sync(0xffffffffu, listed, o);
	}
	if ((threadIdx.x & 31) == 0) {
		atomicAdd(&counts[0], dec);
		atomicAdd(&counts[1], bad);
		atomicAdd(&counts[2], listed);
	}
}

bool debug_expf_check(uint32_t first, uint32_t count, unsigned long long* out, float* band, std::string& err)
{
	ExpExceptions T;
	if (!exp_exceptions_for_device(&T, nullptr, err)) return false;
	if (band) *band = T.band;
	unsigned long long* d = nullptr;
	if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) { err = "cudaMalloc"; return false; }
	cudaMemset(d, 0, 3 * sizeof(unsigned long long));
	if (count > 0) k_expf_check<<<1216, 256>>>(T, first, count, d);
	cudaError_t e = cudaMemcpy(out, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
	cudaFree(d);
	if (e != cudaSuccess) { err = cudaGetErrorString(e); return false; }
	return true;
}

}  // namespace umans
