// ORCA velocities without any allocation.
//
// Some callers of this library cannot allocate GPU memory when they need a
// result: a host application that hands out all device memory through its
// own pool at start-up and forbids cudaMalloc afterwards (game engines and
// simulators embedding the crowd step in a frame loop), or code that runs
// while another component holds the device allocator.  For them this file
// provides one entry point that computes, for agents whose data the caller
// already keeps on the device, the velocity the ORCA policy would choose
// this step, using only memory that exists for the lifetime of the library:
// the ORCA line buffers live in a file-scope __device__ array.
//
// Limits and behaviour:
//  * the scratch array holds NOALLOC_WARPS x 2 x NOALLOC_MAX_LINES lines
//    (1 MiB); the kernel always runs NOALLOC_WARPS warps and each warp owns a
//    fixed slice, so the number of agents is unbounded but a neighbour list
//    may use at most NOALLOC_MAX_LINES entries (nbr_cap <= 128);
//  * every call shares the array, which keeps the last call's contents.  The
//    line buffers are written before they are read; the status word is
//    cleared at the start of every call.  Calls that overlap on the GPU (two
//    streams, or two threads with different streams) race on the array and on
//    the status word: serialise them;
//  * the host name of the array is not a device address; its device address
//    is taken once per device with cudaGetSymbolAddress, with that device
//    current, on the first call on that device;
//  * every call reads the status word back and synchronises `stream`, so it
//    must not be called while that stream is being captured into a graph;
//  * neighbour indices outside [0, n) are skipped and reported (status bit
//    2), never read;
//  * infinite worlds only: neighbours are indices into the caller's arrays,
//    without wrap-around offsets.
#include <cstdio>
#include <cstdarg>
#include <mutex>

#include <cuda_runtime.h>

#include "costs.cuh"
#include "orca.cuh"

namespace umans {

constexpr int NOALLOC_WARPS = 256;
constexpr int NOALLOC_MAX_LINES = 128;

static __device__ __align__(256) float4 g_noalloc_lines[NOALLOC_WARPS * 2 * NOALLOC_MAX_LINES];
static __device__ __align__(256) int g_noalloc_status;

// Policy::ComputeNewVelocity (policy.cpp:43-76) for a policy whose only cost
// is ORCA with the global method: ORCA::GetGlobalMinimum (ORCA.cpp:88-95),
// lines from Solver::createAgentOrcaLines (ORCASolver.cpp:96-171).
__global__ void __launch_bounds__(128) k_orca_noalloc(
	int n, const float2* __restrict__ pos, const float2* __restrict__ vel, const float2* __restrict__ pref,
	const float* __restrict__ radius, const float* __restrict__ max_speed, const float* __restrict__ max_accel,
	const int* __restrict__ nbr_index, const float* __restrict__ nbr_d2, const int* __restrict__ nbr_count,
	int cap, float range, float tH, float dt, float relax, float2* __restrict__ out, float4* scratch, int* status)
{
	const int lane = threadIdx.x & 31;
	const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
	float4* lines = scratch + (size_t)gw * 2 * NOALLOC_MAX_LINES;
	float4* proj = lines + NOALLOC_MAX_LINES;
	const float maxDistSq = range * range;
	for (int i = gw; i < n; i += NOALLOC_WARPS) {
		const float2 p = pos[i], v = vel[i], pv = pref[i];
		const float r = radius[i], ms = max_speed[i], ma = max_accel[i];
		int K = nbr_count[i];
		if (K > cap) {
			if (lane == 0) atomicOr(status, 1);
			K = cap;
		}
		if (K < 0) K = 0;
		float2 nv = V(0, 0);
		if (!viszero(pv)) {
			int nl = 0;
			for (int base = 0; base < K; base += 32) {
				const int k = base + lane;
				bool in = k < K && nbr_d2[(size_t)i * cap + k] <= maxDistSq;
				const int j = in ? nbr_index[(size_t)i * cap + k] : 0;
				if (in && (j < 0 || j >= n)) {   // a stale or corrupt list: skip the entry
					atomicOr(status, 2);
					in = false;
				}
				float4 o = make_float4(0, 0, 0, 0);
				if (in) {
					const float2 relPos = vsub(pos[j], p);
					const float2 relVel = vsub(v, vel[j]);
					const float distSq = vsq(relPos);
					const float cR = r + radius[j];
					const float cRSq = cR * cR;
					float2 dir, u;
					if (distSq > cRSq) {
						const float2 w = vsub(relVel, vdiv(relPos, tH));
						const float wLenSq = vsq(w);
						const float dp1 = vdot(w, relPos);
						if (dp1 < 0.0f && dp1 * dp1 > cRSq * wLenSq) {
							const float wLen = sqrtf(wLenSq);
							const float2 unitW = vdiv(w, wLen);
							dir = V(unitW.y, -unitW.x);
							u = vmul(unitW, cR / tH - wLen);
						} else {
							const float leg = sqrtf(distSq - cRSq);
							if (det2(relPos, w) > 0.0f)
								dir = vdiv(V(relPos.x * leg - relPos.y * cR, relPos.x * cR + relPos.y * leg), distSq);
							else
								dir = vdiv(vmul(V(relPos.x * leg + relPos.y * cR, -relPos.x * cR + relPos.y * leg), -1), distSq);
							u = vsub(vmul(dir, vdot(relVel, dir)), relVel);
						}
					} else {
						const float2 w = vsub(relVel, vdiv(relPos, dt));
						const float wLen = vsq(w);   // sic: ORCASolver.cpp:161
						const float2 unitW = vdiv(w, wLen);
						dir = V(unitW.y, -unitW.x);
						u = vmul(unitW, cR / dt - wLen);
					}
					const float2 pt = vadd(v, vmul(u, 0.5f));
					o = make_float4(pt.x, pt.y, dir.x, dir.y);
				}
				const unsigned m = __ballot_sync(0xffffffffu, in);
				if (in) lines[nl + __popc(m & ((1u << lane) - 1u))] = o;
				nl += __popc(m);
			}
			__syncwarp();
			float2 best;
			const int fail = lp2(lines, nl, ms, pv, false, &best, lane);
			if (fail < nl) lp3(lines, nl, fail, ms, &best, proj, lane);
			float2 acc = vdiv(vsub(best, v), fmaxr(relax, dt));
			acc = vclamp(acc, ma);
			nv = vclamp(vadd(v, vmul(acc, dt)), ms);
		}
		if (lane == 0) out[i] = nv;
		__syncwarp();
	}
}

namespace {
struct Symbols {
	float4* lines = nullptr;
	int* status = nullptr;
	bool ready = false;
};
constexpr int MAX_DEVICES = 64;
Symbols g_syms[MAX_DEVICES];
std::mutex g_sym_mutex;
thread_local char g_err[256];   // per host thread, as the handle API's error flag

int set_error(int code, const char* fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
	va_end(ap);
	return code;
}
}  // namespace

const char* noalloc_last_error() { return g_err; }

int orca_velocities_noalloc(int n, const float* pos, const float* vel, const float* pref, const float* radius,
                            const float* max_speed, const float* max_accel, const int* nbr_index,
                            const float* nbr_dist2, const int* nbr_count, int nbr_cap, float range,
                            float time_horizon, float dt, float relaxation_time, float* new_vel, void* stream)
{
	if (n < 0) return set_error(1, "negative agent count %d", n);
	if (nbr_cap < 0 || nbr_cap > NOALLOC_MAX_LINES)
		return set_error(1, "neighbour capacity %d exceeds the %d ORCA lines per agent of the static scratch",
		                 nbr_cap, NOALLOC_MAX_LINES);
	if (n == 0) return 0;
	if (!pos || !vel || !pref || !radius || !max_speed || !max_accel || !new_vel ||
	    (nbr_cap > 0 && (!nbr_index || !nbr_dist2)) || !nbr_count)
		return set_error(1, "null device pointer");
	if (!(dt > 0) || !(time_horizon > 0)) return set_error(1, "dt and time_horizon must be positive");
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return set_error(3, "no usable CUDA device");
	Symbols& S = g_syms[dev];
	{
		std::lock_guard<std::mutex> lk(g_sym_mutex);
		if (!S.ready) {
			cudaError_t e1 = cudaGetSymbolAddress((void**)&S.lines, g_noalloc_lines);
			cudaError_t e2 = cudaGetSymbolAddress((void**)&S.status, g_noalloc_status);
			if (e1 != cudaSuccess || e2 != cudaSuccess)
				return set_error(3, "cudaGetSymbolAddress: %s", cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
			S.ready = true;
		}
	}
	cudaStream_t st = (cudaStream_t)stream;
	// an error left by the caller's earlier work is reported as such, not as
	// this call's launch failure
	cudaError_t e = cudaPeekAtLastError();
	if (e != cudaSuccess) return set_error(3, "a CUDA error from earlier work is pending: %s", cudaGetErrorString(e));
	e = cudaMemsetAsync(S.status, 0, sizeof(int), st);
	if (e != cudaSuccess) return set_error(3, "cudaMemsetAsync: %s", cudaGetErrorString(e));
	k_orca_noalloc<<<NOALLOC_WARPS / 4, 128, 0, st>>>(
		n, (const float2*)pos, (const float2*)vel, (const float2*)pref, radius, max_speed, max_accel, nbr_index,
		nbr_dist2, nbr_count, nbr_cap, range, time_horizon, dt, relaxation_time, (float2*)new_vel, S.lines, S.status);
	e = cudaGetLastError();
	if (e != cudaSuccess) return set_error(3, "kernel launch: %s", cudaGetErrorString(e));
	int hs = 0;
	e = cudaMemcpyAsync(&hs, S.status, sizeof(int), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (e != cudaSuccess) return set_error(3, "%s", cudaGetErrorString(e));
	if (hs & 2) return set_error(4, "a neighbour index lies outside [0, n); those entries were skipped");
	if (hs) return set_error(4, "a neighbour count exceeds nbr_cap; those lists were truncated");
	return 0;
}

}  // namespace umans
