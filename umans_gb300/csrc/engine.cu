// GB300 step engine: the per-step agent update of WorldBase::DoStep
// (src/Engine/core/worldBase.cpp:79-128) as a short kernel sequence.
//
//   k_bbox / k_grid     bounding box (infinite world) -> grid parameters
//   k_count             cell of every agent, per-cell histogram
//                       (warp-aggregated atomics via __match_any_sync)
//   k_scan_*            exclusive prefix sum of the histogram (3 passes)
//   k_scatter           counting-sort scatter into cell-sorted copies of
//                       position / velocity / preferred velocity / radius,
//                       computing the preferred velocity (agent.cpp:52-59)
//   k_agent             one warp per agent, agents in cell order:
//                         neighbour query (kd-tree radius search semantics,
//                         AgentKDTree.cpp:35-59, worldToric.cpp:32-79),
//                         contact forces (policy.cpp:107-141),
//                         velocity optimisation (policy.cpp:43-105),
//                         integration + toric wrap (agent.cpp:71-93,
//                         worldToric.cpp:81-108).
//
// Phases 2-6 of DoStep only read state that earlier phases finished and only
// write per-agent state, so they fuse into k_agent: every neighbour read goes
// to the cell-sorted copies made by k_scatter, every write to the agent's own
// slot.
#include "engine.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <set>

#include "costs.cuh"
#include "orca.cuh"
#include "adjoint.cuh"

namespace umans {

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { err_ = std::string(#x) + ": " + cudaGetErrorString(e_); return false; } } while (0)

static const uint32_t LCG_M = 2147483647u;   // minstd_rand0 modulus
static const uint32_t LCG_A = 16807u;

struct DevState {
	int n, nscen;
	const ScenDesc* scen;   // [nscen]
	int* agent_scen;        // [n] scenario of each agent, list order
	int* cell_base;         // [nscen + 1]: first cell of each scenario's grid, then the total
	float2 *pos, *vel, *goal, *view, *vwf, *pref;
	float4* prm;
	int *pol, *id;
	uint32_t* rng;
	float2 *sP, *sV;
	float4* sB;
	float4* sE;          // cell order: normalised preferred velocity, speed (SocialForces), radius
	int *sSlot, *sId;
	int *cell, *cnt, *start, *blocksum;   // cnt: per-cell histogram, zero between steps
	unsigned* ticket;       // blocks of k_count_scan done (zero between launches)
	unsigned* gbar;         // k_grid_coop's barrier: arrivals, generation
	GridParams* grid;       // [nscen]
	unsigned* bbox;         // [4 * nscen]
	// profiling only (else null): Karamouzas samples inside the window, pairs
	// swept per window sample, agents through that path
	unsigned long long* counters;
	int* status;
	const PolicyDesc* pols;
	const SampleEntry* table;
	const uint32_t* lcgpow;
	float4* scratch;
	int maxnb, total_warps, max_cells;   // max_cells: capacity of the cell arrays (all scenarios)
	int t_begin, t_end;   // cell-sorted agents this k_agent launch updates
	const float4* edges;  // obstacle edges of all scenarios (ScenDesc::edge_off)
	const int* og_start;  // edge grids (ScenDesc::og_*): cell starts,
	const int2* og_items; // items (global edge index, cell x),
	const int4* og_ecell; // per global edge its cell range (x0, y0, x1, y1)
	uint32_t* obs_list;   // per warp: max_obs entries of the agent's obstacle list
	int max_obs;
	const int* scen_order;   // [nscen]: scenarios in cell-space order (grouped by kernel)
	int sched;            // agent-to-warp schedule: 0 interleaved, 1 contiguous blocks, 2 work list
	unsigned* work;       // schedule 2: this launch's tile counter and finished-warp count (zero between launches)
	float cells_per_range;
	ExpExceptions expx;   // host-expf exception table
	// differentiable form: neighbour lists recorded during a forward step
	// (list-order slot of the neighbour | displacement group << 28), and the
	// adjoint buffers of k_adjoint
	uint32_t* tape_list;  // [n * maxnb] or null
	int* tape_cnt;        // [n]
	const float2 *a_pos, *a_vel;        // state at the start of the step being reversed
	const float2 *lam_out_p, *lam_out_v;
	float2 *lam_in_p, *lam_in_v;
	float2* tape_acc;     // [n]: acceleration before the clamp (gradient method)
	float4* adj_nb;       // [n]: Eb, 1/|goal - pos|, speed (k_adj_prep)
	float* dparams;       // [nscen * 4]: dL/d(V0, sigma, k, tau0)
	int* slot_of_id;      // id -> list slot, -1 when absent
	int id_bound;         // size of slot_of_id
	AgentRecord* io;      // staging for AgentData exchange
	// neighbour-list dump (tests)
	int *dump_ids, *dump_cnt;
	float* dump_d2;
	int dump_cap;
};

// ------------------------------------------------------------------------
// grid build
// ------------------------------------------------------------------------
__device__ __forceinline__ unsigned f2o(float f)
{
	unsigned u = __float_as_uint(f);
	return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(unsigned u)
{
	return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// bounding box of the agents of each infinite-world scenario
__device__ __forceinline__ void bbox_one(const DevState& S, int i)
{
	const int s = S.agent_scen[i];
	if (S.scen[s].world == W_TORIC) return;
	const float2 p = S.pos[i];
	const unsigned peers = __match_any_sync(__activemask(), s);
	const unsigned a = __reduce_min_sync(peers, f2o(p.x)), b = __reduce_min_sync(peers, f2o(p.y));
	const unsigned c = __reduce_max_sync(peers, f2o(p.x)), d = __reduce_max_sync(peers, f2o(p.y));
	if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
		unsigned* B = S.bbox + 4 * s;
		atomicMin(&B[0], a); atomicMin(&B[1], b);
		atomicMax(&B[2], c); atomicMax(&B[3], d);
	}
}
__global__ void k_bbox(DevState S)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < S.n) bbox_one(S, i);
}

// grid of scenario s (origin, cell size, counts) from its bounding box, which
// is reset for the next step; returns the scenario's cell count
__device__ int grid_params(const DevState& S, int s)
{
	const ScenDesc sd = S.scen[s];
	unsigned* B = S.bbox + 4 * s;
	float x0, y0, ex, ey;
	if (sd.world == W_TORIC) {
		x0 = -0.5f * sd.width; y0 = -0.5f * sd.height; ex = sd.width; ey = sd.height;
	} else {
		x0 = o2f(__ldcg(&B[0])); y0 = o2f(__ldcg(&B[1]));
		ex = o2f(__ldcg(&B[2])) - x0; ey = o2f(__ldcg(&B[3])) - y0;
		if (sd.n == 0) { x0 = y0 = 0; ex = ey = 1; }
	}
	B[0] = B[1] = f2o(FLT_MAX);
	B[2] = B[3] = f2o(-FLT_MAX);
	if (!isfinite(x0) || !isfinite(y0) || !isfinite(ex) || !isfinite(ey)) {
		atomicOr(S.status, ST_GRID_OVERFLOW);
		x0 = y0 = 0; ex = ey = 1;
	}
	float cs = sd.max_range / S.cells_per_range;
	if (!(cs >= 1e-3f)) cs = 1e-3f;
	// +2 per axis: nx, ny below come from float divisions that may round up
	while (((double)ex / cs + 2.0) * ((double)ey / cs + 2.0) > (double)sd.max_cells) cs *= 2.0f;
	GridParams g;
	g.x0 = x0; g.y0 = y0; g.cs = cs; g.inv_cs = 1.0f / cs;
	g.nx = (int)(ex / cs) + 1; g.ny = (int)(ey / cs) + 1;
	g.ncells = g.nx * g.ny; g.pad = 0;
	S.grid[s] = g;
	return g.ncells;
}

// One block: grid parameters of every scenario, then the exclusive scan of
// their cell counts into cell_base (scenario grids are concatenated in
// scen_order, which groups scenarios by the k_agent specialisation they use,
// so that each group's agents form one range of the cell-sorted arrays).
__global__ void __launch_bounds__(1024) k_grid(DevState S)
{
	const int ns = S.nscen;
	const int per = (ns + blockDim.x - 1) / blockDim.x;
	const int s0 = threadIdx.x * per;
	int local = 0;
	for (int k = 0; k < per && s0 + k < ns; ++k) {
		const int s = S.scen_order[s0 + k];
		const int nc = grid_params(S, s);
		S.cell_base[s] = nc;
		local += nc;
	}
	__shared__ int tot[1024];
	tot[threadIdx.x] = local;
	__syncthreads();
	for (int o = 1; o < (int)blockDim.x; o <<= 1) {
		const int v = threadIdx.x >= o ? tot[threadIdx.x - o] : 0;
		__syncthreads();
		tot[threadIdx.x] += v;
		__syncthreads();
	}
	int run = tot[threadIdx.x] - local;
	for (int k = 0; k < per && s0 + k < ns; ++k) {
		const int s = S.scen_order[s0 + k];
		const int c = S.cell_base[s];
		S.cell_base[s] = run;
		run += c;
	}
	if (threadIdx.x == blockDim.x - 1) S.cell_base[ns] = tot[threadIdx.x];
}

__device__ __forceinline__ int cell_coord(float v, float v0, float inv, int nmax)
{
	const float f = (v - v0) * inv;
	int c = (f >= 0.0f) ? (int)fminf(f, 2.0e9f) : 0;   // NaN -> 0
	return c >= nmax ? nmax - 1 : c;
}

// cell of agent i (grid g, cells of its scenario from cb) and its histogram count
__device__ __forceinline__ void count_one(const DevState& S, int i, const GridParams& g, int cb)
{
	const float2 p = S.pos[i];
	const int c = cb + cell_coord(p.y, g.y0, g.inv_cs, g.ny) * g.nx + cell_coord(p.x, g.x0, g.inv_cs, g.nx);
	S.cell[i] = c;
	const unsigned peers = __match_any_sync(__activemask(), c);
	if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&S.cnt[c], __popc(peers));
}
__global__ void k_count(DevState S)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= S.n) return;
	const int sc = S.agent_scen[i];
	count_one(S, i, S.grid[sc], S.cell_base[sc]);
}

// exclusive scan of cnt[0..ncells) into start in 3 passes; 1024 cells per
// block (k_scatter takes the counts back to zero)
constexpr int SCAN_BLOCK = 256, SCAN_PER_BLOCK = 1024;

__global__ void k_scan_reduce(DevState S)
{
	const int nc = S.cell_base[S.nscen];
	const int base = blockIdx.x * SCAN_PER_BLOCK;
	if (base >= nc) return;
	int s = 0;
	for (int k = threadIdx.x; k < SCAN_PER_BLOCK; k += SCAN_BLOCK) {
		const int c = base + k;
		if (c < nc) s += S.cnt[c];
	}
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	__shared__ int ws[SCAN_BLOCK / 32];
	if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		int t = 0;
		for (int w = 0; w < SCAN_BLOCK / 32; ++w) t += ws[w];
		S.blocksum[blockIdx.x] = t;
	}
}

__global__ void k_scan_top(DevState S)
{
	// one block of 1024 threads; exclusive scan of the block sums in place
	const int nb = (S.cell_base[S.nscen] + SCAN_PER_BLOCK - 1) / SCAN_PER_BLOCK;
	const int per = (nb + 1023) / 1024;
	const int b0 = threadIdx.x * per;
	int local = 0;
	for (int k = 0; k < per; ++k) if (b0 + k < nb) local += S.blocksum[b0 + k];
	__shared__ int tot[1024];
	tot[threadIdx.x] = local;
	__syncthreads();
	for (int o = 1; o < 1024; o <<= 1) {
		int v = threadIdx.x >= o ? tot[threadIdx.x - o] : 0;
		__syncthreads();
		tot[threadIdx.x] += v;
		__syncthreads();
	}
	int run = tot[threadIdx.x] - local;
	for (int k = 0; k < per; ++k) {
		if (b0 + k < nb) {
			const int v = S.blocksum[b0 + k];
			S.blocksum[b0 + k] = run;
			run += v;
		}
	}
}

__global__ void k_scan_down(DevState S)
{
	const int nc = S.cell_base[S.nscen];
	const int base = blockIdx.x * SCAN_PER_BLOCK;
	if (base >= nc) return;
	// each thread owns 4 consecutive cells
	const int c0 = base + threadIdx.x * 4;
	int v[4], s = 0;
	for (int k = 0; k < 4; ++k) { v[k] = (c0 + k < nc) ? S.cnt[c0 + k] : 0; s += v[k]; }
	__shared__ int ts[SCAN_BLOCK];
	ts[threadIdx.x] = s;
	__syncthreads();
	for (int o = 1; o < SCAN_BLOCK; o <<= 1) {
		int x = threadIdx.x >= o ? ts[threadIdx.x - o] : 0;
		__syncthreads();
		ts[threadIdx.x] += x;
		__syncthreads();
	}
	int run = S.blocksum[blockIdx.x] + ts[threadIdx.x] - s;
	for (int k = 0; k < 4; ++k) {
		const int c = c0 + k;
		if (c < nc) {
			S.start[c] = run;
			run += v[k];
		}
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) S.start[nc] = S.n;
}

// Exclusive scan of cnt[0..nc) by one block through shared memory (sm holds
// nc + nc/32 ints; the index is padded by one word per 32 so that per-thread
// runs of cells fall in different banks): coalesced loads, eight in flight
// per thread, then per thread a contiguous run of cells summed, a block scan
// of the run sums, the runs rewritten with their prefixes, and a coalesced
// write of start.  (The histogram itself is left as it is: k_scatter counts
// every cell back down to zero.)
constexpr int SCAN_SMEM_MAX_CELLS = 49152;
__host__ __device__ constexpr size_t scan_smem_bytes(int cells) { return sizeof(int) * ((size_t)cells + cells / 32 + 1); }
__device__ __forceinline__ int scan_pad(int c) { return c + (c >> 5); }
__device__ void block_scan_cells(const DevState& S, int nc, int* sm)
{
	const int tid = threadIdx.x, nt = blockDim.x;
	const int* __restrict__ cnt = S.cnt;
	for (int c0 = tid; c0 < nc; c0 += 8 * nt) {
		int v[8];
#pragma unroll
		for (int k = 0; k < 8; ++k) {
			const int c = c0 + k * nt;
			v[k] = c < nc ? __ldcg(cnt + c) : 0;
		}
#pragma unroll
		for (int k = 0; k < 8; ++k) {
			const int c = c0 + k * nt;
			if (c < nc) sm[scan_pad(c)] = v[k];
		}
	}
	__syncthreads();
	const int L = (nc + nt - 1) / nt;
	const int c0 = min(nc, tid * L), c1 = min(nc, c0 + L);
	int s = 0;
	for (int c = c0; c < c1; ++c) s += sm[scan_pad(c)];
	const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
	int incl = s;
	for (int o = 1; o < 32; o <<= 1) {
		const int u = __shfl_up_sync(0xffffffffu, incl, o);
		if (lane >= o) incl += u;
	}
	__shared__ int wt[32];
	if (lane == 31) wt[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		const int v = lane < nw ? wt[lane] : 0;
		int w = v;
		for (int o = 1; o < 32; o <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, w, o);
			if (lane >= o) w += u;
		}
		if (lane < nw) wt[lane] = w - v;
	}
	__syncthreads();
	int run = wt[warp] + incl - s;
	for (int c = c0; c < c1; ++c) {
		const int v = sm[scan_pad(c)];
		sm[scan_pad(c)] = run;
		run += v;
	}
	__syncthreads();
	int* __restrict__ start = S.start;
	for (int c = tid; c < nc; c += nt) start[c] = sm[scan_pad(c)];
	if (tid == 0) start[nc] = S.n;
}

// One block, grids of at most `cap` (<= SCAN_SMEM_MAX_CELLS) cells.
__global__ void __launch_bounds__(1024) k_scan_smem(DevState S, int cap)
{
	extern __shared__ int sm[];
	const int nc = S.cell_base[S.nscen];
	if (nc > cap) {   // cannot happen: cap bounds every grid the engine builds
		if (threadIdx.x == 0) atomicOr(S.status, ST_GRID_OVERFLOW);
		return;
	}
	block_scan_cells(S, nc, sm);
}

// The histogram and, in the last block to finish, the scan: one launch for
// grids whose cell count is fixed and at most `cap` cells (toric worlds).
// Each block counts its agents, fences, and takes a ticket; the block that
// takes the last ticket sees every other block's counts in L2 and scans them
// (no block waits for another).
__global__ void __launch_bounds__(1024) k_count_scan(DevState S, int cap)
{
	extern __shared__ int sm[];
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < S.n) {
		const int sc = S.agent_scen[i];
		count_one(S, i, S.grid[sc], S.cell_base[sc]);
	}
	__threadfence();
	__syncthreads();
	__shared__ bool last;
	if (threadIdx.x == 0) {
		const unsigned t = atomicAdd(S.ticket, 1u);
		last = t == gridDim.x - 1;
		if (last) *S.ticket = 0u;   // for the next launch
	}
	__syncthreads();
	if (!last) return;
	__threadfence();
	const int nc = S.cell_base[S.nscen];
	if (nc > cap) {
		if (threadIdx.x == 0) atomicOr(S.status, ST_GRID_OVERFLOW);
		return;
	}
	block_scan_cells(S, nc, sm);
}

// Barrier of all blocks of a cooperative launch (every block resident): an
// arrival count and a generation word.  The last block to arrive resets the
// count and advances the generation.  The wait is bounded: after GBAR_SPINS
// polls the block records ST_GRID_BARRIER and goes on (the host then reports
// an error).  That cannot happen while every block is resident, which the
// cooperative launch guarantees.
constexpr int GBAR_SPINS = 1 << 22;
__device__ __forceinline__ void grid_barrier(const DevState& S)
{
	__syncthreads();
	if (threadIdx.x == 0) {
		volatile unsigned* gen = S.gbar + 1;
		const unsigned g = *gen;
		__threadfence();
		if (atomicAdd(S.gbar, 1u) == gridDim.x - 1) {
			S.gbar[0] = 0u;
			__threadfence();
			atomicAdd(S.gbar + 1, 1u);
		} else {
			int spins = 0;
			while (*gen == g) {
				if (++spins > GBAR_SPINS) {
					atomicOr(S.status, ST_GRID_BARRIER);
					break;
				}
				__nanosleep(32);
			}
		}
		__threadfence();
	}
	__syncthreads();
}

// The same exclusive scan in one block, for grids of at most
// SCAN_SINGLE_MAX_CELLS cells (one launch instead of three): each warp scans
// a contiguous range of cells in coalesced chunks of 32, after a first pass
// that sums the warps' ranges.
constexpr int SCAN_SINGLE_MAX_CELLS = 1 << 17;
__global__ void __launch_bounds__(1024) k_scan_single(DevState S)
{
	const int nc = S.cell_base[S.nscen];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const int per = (((nc + nw - 1) / nw) + 31) & ~31;
	const int w0 = min(nc, warp * per), w1 = min(nc, w0 + per);
	int s = 0;
	for (int c = w0 + lane; c < w1; c += 32) s += S.cnt[c];
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	__shared__ int wt[32];
	if (lane == 0) wt[warp] = s;
	__syncthreads();
	if (warp == 0) {
		const int v = lane < nw ? wt[lane] : 0;
		int incl = v;
		for (int o = 1; o < 32; o <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, incl, o);
			if (lane >= o) incl += u;
		}
		if (lane < nw) wt[lane] = incl - v;
	}
	__syncthreads();
	// the loads do not depend on the running total: distinct arrays, so that
	// they can be issued ahead of the stores
	const int* __restrict__ cnt = S.cnt;
	int* __restrict__ start = S.start;
	int run = wt[warp];
#pragma unroll 4
	for (int base = w0; base < w1; base += 32) {
		const int c = base + lane;
		const int v = c < w1 ? __ldcg(cnt + c) : 0;
		int incl = v;
		for (int o = 1; o < 32; o <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, incl, o);
			if (lane >= o) incl += u;
		}
		if (c < w1) start[c] = run + incl - v;
		run += __shfl_sync(0xffffffffu, incl, 31);
	}
	if (threadIdx.x == 0) S.start[nc] = S.n;
}

__device__ __forceinline__ void scatter_one(const DevState& S, int i)
{
	const int c = S.cell[i];
	const unsigned act = __activemask();
	const unsigned peers = __match_any_sync(act, c);
	const int lane = threadIdx.x & 31;
	const int leader = __ffs(peers) - 1;
	// the cell is filled from its top down: the histogram count is taken back
	// by each agent placed, so it is all-zero again for the next step
	int top = 0;
	if (lane == leader) top = atomicSub(&S.cnt[c], __popc(peers));
	top = __shfl_sync(peers, top, leader);
	const int t = __ldcg(S.start + c) + top - __popc(peers) + __popc(peers & ((1u << lane) - 1u));
	const float2 p = S.pos[i];
	const float2 g = S.goal[i];
	const float4 prm = S.prm[i];
	// Agent::ComputePreferredVelocity / hasReachedGoal: agent.cpp:52-59, 99-102
	const float2 d = vsub(g, p);
	float2 pv;
	if (vsq(d) <= prm.x * prm.x) pv = V(0, 0);
	else pv = vmul(vnorm(d), prm.y);
	S.pref[i] = pv;
	S.sP[t] = p;
	S.sV[t] = S.vel[i];
	S.sB[t] = make_float4(pv.x, pv.y, prm.x, 0.0f);
	// per-agent terms of SocialForcesAvoidance.cpp:58-59 (vb, Eb), computed once
	// here instead of once per neighbour pair; the same operations, so the
	// same values
	const float2 v = S.vel[i];
	const float2 eb = vnorm(pv);
	S.sE[t] = make_float4(eb.x, eb.y, vmag(v), prm.x);   // w: the radius, for the force pass's single load
	S.sSlot[t] = i;
	S.sId[t] = S.id[i];
}
__global__ void k_scatter(DevState S)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < S.n) scatter_one(S, i);
}

// The whole grid build of a static grid in one cooperative launch: the
// histogram (blocks striding over the agents), a barrier, each block's sum of
// its stretch of cells, a barrier, each block's exclusive scan of its stretch
// (after the sums of the stretches before it), a barrier, the scatter.  No
// one-block scan and no launch in between.
__global__ void __launch_bounds__(1024) k_grid_coop(DevState S)
{
	const int n = S.n, nt = blockDim.x, tid = threadIdx.x;
	const int stride = gridDim.x * nt;
	for (int i = blockIdx.x * nt + tid; i < n; i += stride) {
		// the scatter's inputs, fetched into L2 while the count and scan run
		asm volatile("prefetch.global.L2 [%0];" ::"l"(S.vel + i));
		asm volatile("prefetch.global.L2 [%0];" ::"l"(S.goal + i));
		asm volatile("prefetch.global.L2 [%0];" ::"l"(S.prm + i));
		asm volatile("prefetch.global.L2 [%0];" ::"l"(S.id + i));
		const int sc = S.agent_scen[i];
		count_one(S, i, S.grid[sc], S.cell_base[sc]);
	}
	grid_barrier(S);
	const int nc = S.cell_base[S.nscen];
	const int seg = (nc + gridDim.x - 1) / gridDim.x;
	const int c0 = min(nc, (int)blockIdx.x * seg), c1 = min(nc, c0 + seg);
	__shared__ int red[32];
	const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
	// block sum of the stretch
	int s = 0;
	for (int c = c0 + tid; c < c1; c += nt) s += __ldcg(S.cnt + c);
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	if (lane == 0) red[warp] = s;
	__syncthreads();
	if (tid == 0) {
		int t = 0;
		for (int w = 0; w < nw; ++w) t += red[w];
		S.blocksum[blockIdx.x] = t;
	}
	grid_barrier(S);
	// the sums of the stretches before this one
	int before = 0;
	for (int b = tid; b < (int)blockIdx.x; b += nt) before += __ldcg(S.blocksum + b);
	for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
	__syncthreads();
	if (lane == 0) red[warp] = before;
	__syncthreads();
	if (warp == 0) {
		int v = lane < nw ? red[lane] : 0;
		for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
		if (lane == 0) red[0] = v;
	}
	__syncthreads();
	int run = red[0];
	__syncthreads();
	// exclusive scan of the stretch, 1024 cells per round
	for (int base = c0; base < c1; base += nt) {
		const int c = base + tid;
		const int v = c < c1 ? __ldcg(S.cnt + c) : 0;
		int incl = v;
		for (int o = 1; o < 32; o <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, incl, o);
			if (lane >= o) incl += u;
		}
		if (lane == 31) red[warp] = incl;
		__syncthreads();
		if (warp == 0) {
			const int wv = lane < nw ? red[lane] : 0;
			int w = wv;
			for (int o = 1; o < 32; o <<= 1) {
				const int u = __shfl_up_sync(0xffffffffu, w, o);
				if (lane >= o) w += u;
			}
			if (lane < nw) red[lane] = w - wv;
		}
		__syncthreads();
		if (c < c1) S.start[c] = run + red[warp] + incl - v;
		const int tot = __shfl_sync(0xffffffffu, incl, 31);
		__syncthreads();
		// the round's total: the last warp's offset plus its own total
		if (warp == nw - 1 && lane == 31) red[0] = red[nw - 1] + tot;
		__syncthreads();
		run += red[0];
		__syncthreads();
	}
	if (blockIdx.x == 0 && tid == 0) S.start[nc] = n;
	grid_barrier(S);
	for (int i = blockIdx.x * nt + tid; i < n; i += stride) scatter_one(S, i);
}

// The whole grid build of a small single-scenario world in one block (the
// same steps as k_bbox .. k_scatter, phases separated by block barriers):
// one launch instead of seven, for worlds whose steps are launch-bound.
// Values written by atomics in one phase are read through L2 (__ldcg).
constexpr int SMALL_MAX_AGENTS = 4096, SMALL_MAX_CELLS = 32768;
__global__ void __launch_bounds__(1024) k_build_small(DevState S)
{
	const int n = S.n, tid = threadIdx.x, nt = blockDim.x;
	for (int i = tid; i < n; i += nt) bbox_one(S, i);
	__syncthreads();
	__shared__ GridParams g;
	__shared__ int ncs;
	if (tid == 0) {
		const int nc = grid_params(S, 0);
		S.cell_base[0] = 0;
		S.cell_base[1] = nc;
		g = S.grid[0];
		ncs = nc;
	}
	__syncthreads();
	for (int i = tid; i < n; i += nt) count_one(S, i, g, 0);
	__syncthreads();
	// exclusive scan of the histogram: per thread a run of cells, then the
	// block's thread sums
	const int nc = ncs;
	const int per = (nc + nt - 1) / nt;
	const int c0 = min(nc, tid * per), c1 = min(nc, c0 + per);
	int local = 0;
	for (int c = c0; c < c1; ++c) local += __ldcg(&S.cnt[c]);
	__shared__ int tot[1024];
	tot[tid] = local;
	__syncthreads();
	for (int o = 1; o < nt; o <<= 1) {
		const int v = tid >= o ? tot[tid - o] : 0;
		__syncthreads();
		tot[tid] += v;
		__syncthreads();
	}
	int run = tot[tid] - local;
	for (int c = c0; c < c1; ++c) {
		const int v = __ldcg(&S.cnt[c]);
		S.start[c] = run;
		run += v;
	}
	if (tid == 0) S.start[nc] = n;
	__syncthreads();
	for (int i = tid; i < n; i += nt) scatter_one(S, i);
}

// ------------------------------------------------------------------------
// neighbour query (warp-cooperative)
// ------------------------------------------------------------------------
struct WarpLists {
	uint32_t* ref;   // (displacement group << 28) | cell-sorted index
	float* key;      // sort key, then PhantomAgent::distSqr
	int* nid;        // scratch: per-neighbour x terms of the ordered force sums
	float* aux;      // per-neighbour y terms
};

// (key, id) order; ids are read from the cell-sorted copy when keys tie
__device__ __forceinline__ bool nb_less(const DevState& S, const WarpLists& L, int a, int b)
{
	const float ka = L.key[a], kb = L.key[b];
	if (ka != kb) return ka < kb;
	return S.sId[L.ref[a] & 0x0FFFFFFFu] < S.sId[L.ref[b] & 0x0FFFFFFFu];
}
__device__ __forceinline__ void nb_cmpswap(const DevState& S, const WarpLists& L, int lo, int hi)
{
	if (nb_less(S, L, hi, lo)) {
		float k = L.key[lo]; L.key[lo] = L.key[hi]; L.key[hi] = k;
		uint32_t r = L.ref[lo]; L.ref[lo] = L.ref[hi]; L.ref[hi] = r;
	}
}

// ascending bitonic sort of [s, s+len) by (key, id); the network compares
// only i < j pairs with the min going to i, so the missing elements of the
// power-of-two padding behave as +infinity and are simply skipped.
__device__ void warp_sort(const DevState& S, const WarpLists& L, int s, int len, int lane)
{
	if (len <= 1) return;
	int lp = 0;
	while ((1 << lp) < len) ++lp;
	const int halfP = 1 << (lp - 1);   // pairs per stage
	for (int ls = 1; ls <= lp; ++ls) {
		// first step of block size 2^ls: i against its mirror in the block
		const int lh = ls - 1;
		for (int k = lane; k < halfP; k += 32) {
			const int blk = k >> lh, pos = k & ((1 << lh) - 1);
			const int lo = (blk << ls) + pos, hi = (blk << ls) + (1 << ls) - 1 - pos;
			if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
		}
		__syncwarp();
		// half-cleaners with distance 2^lj
		for (int lj = lh - 1; lj >= 0; --lj) {
			for (int k = lane; k < halfP; k += 32) {
				const int lo = ((k >> lj) << (lj + 1)) | (k & ((1 << lj) - 1)), hi = lo + (1 << lj);
				if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
			}
			__syncwarp();
		}
	}
}

// Sort of [s, s+len), len <= 32 * M (M = 1, 2, 4), in registers: each lane
// holds M packed keys (float key bits with the low PB bits replaced by the
// position in the segment; positive floats order like their bit patterns)
// and a shuffle bitonic network sorts them.  The entries (reference and
// full key) are then permuted through registers.  Keys that agree above the low PB
// bits may come out in either order: the near-tie pass that follows
// (relative window 2^(PB-22), twice the 2^(PB-23) truncation) re-orders
// them with the exact double distance and the id.
template <int M>
__device__ __forceinline__ void warp_sort_regs(const WarpLists& L, int s, int len, int lane)
{
	constexpr int PB = (M == 1) ? 5 : (M == 2) ? 6 : 7;
	constexpr uint32_t PMASK = (1u << PB) - 1u;
	uint32_t u[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * 32 + lane;
		u[m] = (i < len) ? ((__float_as_uint(L.key[s + i]) & ~PMASK) | (uint32_t)i) : 0xffffffffu;
	}
	constexpr int P = 32 * M;
#pragma unroll
	for (int size = 2; size <= P; size <<= 1) {
#pragma unroll
		for (int j = size >> 1; j > 0; j >>= 1) {
#pragma unroll
			for (int m = 0; m < M; ++m) {
				const int i = m * 32 + lane;
				const bool up = (i & size) == 0;
				if (j >= 32) {
					const int mm = m ^ (j >> 5);
					if (mm > m) {
						const uint32_t a = u[m], b = u[mm];
						const bool swap = up ? (a > b) : (a < b);
						if (swap) { u[m] = b; u[mm] = a; }
					}
				} else {
					const uint32_t o = __shfl_xor_sync(0xffffffffu, u[m], j);
					const bool lower = (lane & j) == 0;
					// keep the min in the lower position of an ascending pair
					const bool take_min = (lower == up);
					u[m] = take_min ? min(u[m], o) : max(u[m], o);
				}
			}
		}
	}
	float k[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * 32 + lane;
		const int from = s + (int)(u[m] & PMASK);
		k[m] = (i < len) ? L.key[from] : 0.0f;
		u[m] = (i < len) ? L.ref[from] : 0u;
	}
	__syncwarp();
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * 32 + lane;
		if (i < len) {
			L.ref[s + i] = u[m];
			L.key[s + i] = k[m];
		}
	}
	__syncwarp();
}

__device__ __forceinline__ double exact_key(float2 q, float2 c)
{
	// nanoflann L2_Simple_Adaptor<double>::evalMetric (nanoflann.hpp:423-446)
	const double d0 = __dsub_rn((double)q.x, (double)c.x);
	const double d1 = __dsub_rn((double)q.y, (double)c.y);
	return __dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1));
}

// Float keys order the list except within runs of near-equal keys (relative
// gap <= win: 1e-6 after the exact-key sort, 2^-16 or 2^-15 after the
// packed-key register sorts, whose keys are truncated), which lane 0
// re-sorts in the reference's order.  Float keys carry a relative error below
// 2.5e-7 (one rounding of each difference, square and sum), so two keys more
// than 1e-6 apart order as the exact ones do; closer pairs are compared on the
// reference's double distance, then the id.
// insertion sort of the run [r0, r1] (lane 0) in the reference's order
__device__ void sort_run(const DevState& S, const WarpLists& L, int r0, int r1, float2 q)
{
	for (int x = r0 + 1; x <= r1; ++x) {
		const uint32_t rx = L.ref[x];
		const float kx = L.key[x];
		int y = x - 1;
		while (y >= r0) {
			const uint32_t ry = L.ref[y];
			const float ky = L.key[y];
			bool after;   // entry y belongs after entry x
			if (ky - kx > 1e-6f * ky) after = true;
			else if (kx - ky > 1e-6f * kx) after = false;
			else {
				const double dx = exact_key(q, S.sP[rx & 0x0FFFFFFFu]);
				const double dy = exact_key(q, S.sP[ry & 0x0FFFFFFFu]);
				after = dy > dx || (dy == dx && S.sId[ry & 0x0FFFFFFFu] > S.sId[rx & 0x0FFFFFFFu]);
			}
			if (!after) break;
			L.ref[y + 1] = ry; L.key[y + 1] = ky;
			--y;
		}
		L.ref[y + 1] = rx; L.key[y + 1] = kx;
	}
}

__device__ void fix_near_ties(const DevState& S, const WarpLists& L, int s, int e, float2 q, int lane, float win)
{
	// flags of the adjacent pairs (k, k+1) whose keys are within the window,
	// one bit per pair, 32 pairs per word in the (free) aux list.  Runs are
	// the maximal sequences of flagged pairs; re-sorting a run only permutes
	// keys inside it, so all flags can be taken from the keys as sorted.
	unsigned* words = reinterpret_cast<unsigned*>(L.aux);
	const int npairs = e - 1 - s;
	unsigned any = 0;
	for (int w = 0; 32 * w < npairs; ++w) {
		const int k = s + 32 * w + lane;
		bool close = false;
		if (k + 1 < e) {
			const float a = L.key[k], b = L.key[k + 1];
			close = b - a <= win * b;
		}
		const unsigned m = __ballot_sync(0xffffffffu, close);
		if (lane == 0) words[w] = m;
		any |= m;
	}
	if (!any) return;
	__syncwarp();
	if (lane == 0) {
		const int nw = (npairs + 31) / 32;
		int p = 0;   // next pair to look at
		while (p < npairs) {
			// first flagged pair at or after p
			int w = p >> 5;
			unsigned m = words[w] & (~0u << (p & 31));
			while (!m && ++w < nw) m = words[w];
			if (!m) break;
			const int r0 = 32 * w + __ffs(m) - 1;
			// first unflagged pair after it (or the end)
			int u = r0 >> 5;
			unsigned z = ~words[u] & (~0u << (r0 & 31));
			while (!z && ++u < nw) z = ~words[u];
			const int r1 = z ? min(32 * u + __ffs(z) - 1, npairs) : npairs;
			// pairs r0 .. r1-1 flagged: entries r0 .. r1 form the run
			sort_run(S, L, s + r0, s + r1, q);
			p = r1 + 1;
		}
	}
	__syncwarp();
}

// Gathers the neighbour list of the agent at cell-sorted index t.  Returns
// the list length (clamped to maxnb; *overflow set when clamped).  Entries
// are grouped by displacement in the reference's order (worldToric.cpp:61-79)
// and each group is sorted by the reference's double distance, ties by id.
// On return key[] holds PhantomAgent::distSqr (worldBase.h:73-77).
__device__ int gather(const DevState& S, const GridParams& G, int cb, int world, float W, float H, const WarpLists& L,
                      int t, float2 p, float r, int lane, bool* overflow)
{
	int K = 0, K0 = 0;
	const int maxnb = S.maxnb;
	if (!(r > 0)) return 0;   // dist < r*r never holds for r = 0
	const float r2 = r * r;
	const double r2d = (double)r2;
	const float r2lo = r2 * 0.999999f, r2hi = r2 * 1.000001f;
	const unsigned lt = (1u << lane) - 1u;
	for (int g = 0; g < 5; ++g) {
		float2 disp = V(0, 0);
		if (g > 0) {
			if (world != W_TORIC) break;
			bool active;
			// worldToric.cpp:64-76 compares the float p.x - r with the double
			// -0.5*W; -0.5f*W is that value exactly, so the float compare agrees
			if (g == 1) { active = (p.x - r) < -0.5f * W; disp = V(W, 0); }
			else if (g == 2) { active = (p.x + r) > 0.5f * W; disp = V(-W, 0); }
			else if (g == 3) { active = (p.y - r) < -0.5f * H; disp = V(0, H); }
			else { active = (p.y + r) > 0.5f * H; disp = V(0, -H); }
			if (!active) continue;
		}
		const float2 q = vadd(p, disp);
		const int gs = K;
		const int cx0 = cell_coord((q.x - r - G.x0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.nx);
		const int cx1 = cell_coord((q.x + r - G.x0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.nx);
		const int cy0 = cell_coord((q.y - r - G.y0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.ny);
		const int cy1 = cell_coord((q.y + r - G.y0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.ny);
		// rows of cells covering the query square, ROWS at a time: lane k loads
		// the contiguous sorted range of row k, the rows are concatenated and
		// scanned in full 32-lane chunks
		constexpr int ROWS = 8;
		for (int ry = cy0; ry <= cy1; ry += ROWS) {
			const int nr = min(ROWS, cy1 - ry + 1);
			int rs = 0, len = 0;
			if (lane < nr) {
				const int c0 = cb + (ry + lane) * G.nx;
				rs = S.start[c0 + cx0];
				len = S.start[c0 + cx1 + 1] - rs;
			}
			int incl = len;
			for (int o = 1; o < ROWS; o <<= 1) {
				const int v = __shfl_up_sync(0xffffffffu, incl, o);
				if (lane >= o) incl += v;
			}
			// lane k < ROWS holds row k's start in the concatenation (rows past
			// nr are empty and start at the total)
			const int beg = incl - len;
			const int total = __shfl_sync(0xffffffffu, incl, ROWS - 1);
			// two chunks of 32 candidates per pass: both chunks' positions are
			// loaded before either is tested
			for (int base = 0; base < total; base += 64) {
				const int nh = base + 32 < total ? 2 : 1;
				int tt[2];
				float2 cp[2];
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					if (h >= nh) break;
					const int c = base + 32 * h + lane;
					// the last row starting at or before c (binary search over the
					// ROWS starts, held by lanes 0..ROWS-1)
					int r = 0;
#pragma unroll
					for (int step = ROWS / 2; step > 0; step >>= 1)
						if (__shfl_sync(0xffffffffu, beg, r + step) <= c) r += step;
					tt[h] = __shfl_sync(0xffffffffu, rs, r) + (c - __shfl_sync(0xffffffffu, beg, r));
					cp[h] = (c < total && tt[h] != t) ? S.sP[tt[h]] : V(0, 0);
				}
#pragma unroll
				for (int h = 0; h < 2; ++h) {
					if (h >= nh) break;
					const int c = base + 32 * h + lane;
					bool ok = false;
					float d2f = 0;
					if (c < total && tt[h] != t) {
						const float dx = q.x - cp[h].x, dy = q.y - cp[h].y;
						d2f = dx * dx + dy * dy;
						if (d2f < r2lo) ok = true;
						else if (d2f <= r2hi) ok = exact_key(q, cp[h]) < r2d;
					}
					const unsigned m = __ballot_sync(0xffffffffu, ok);
					if (ok) {
						const int idx = K + __popc(m & lt);
						if (idx < maxnb) {
							L.ref[idx] = ((uint32_t)g << 28) | (uint32_t)tt[h];
							L.key[idx] = d2f;
						}
					}
					K += __popc(m);
				}
			}
		}
		if (K > maxnb) { *overflow = true; K = maxnb; }
		if (g == 0) K0 = K;
		__syncwarp();
		const int len = K - gs;
		if (len <= 32) warp_sort_regs<1>(L, gs, len, lane);
		else if (len <= 64) warp_sort_regs<2>(L, gs, len, lane);
		else if (len <= 128) warp_sort_regs<4>(L, gs, len, lane);
		else warp_sort(S, L, gs, len, lane);
		fix_near_ties(S, L, gs, K, q, lane, len <= 64 ? 0x1p-16f : (len <= 128 ? 0x1p-15f : 1e-6f));
	}
	// PhantomAgent position offset = -displacement; distSqr in float.  For
	// the undisplaced group the sort keys are already that value (same
	// operands, same operations), so only displaced entries are recomputed.
	for (int k = K0 + lane; k < K; k += 32) {
		const uint32_t rr = L.ref[k];
		const float2 ph = vadd(S.sP[rr & 0x0FFFFFFFu], group_offset(rr >> 28, W, H));
		L.key[k] = vsq(vsub(p, ph));
	}
	__syncwarp();
	return K;
}

// The edge-grid query of gather_obstacles for one displacement group: the
// cells covering the query square (with a 1% cell margin); an edge is taken
// in the first of them that its own box covers, so once, and the same
// distance test decides; the group's edges are then put in edge (file)
// order.  Appends to out[K..]; returns the new count.
__device__ __forceinline__ int gather_obstacles_grid(const DevState& S, const ScenDesc& sd, float2 q, float r, int g,
                                                  int lane, uint32_t* out, int K)
{
	const float r2 = r * r;
	const unsigned lt = (1u << lane) - 1u;
	const int gs = K;
	const int qx0 = obs_cell((q.x - r - sd.og_x0) * sd.og_inv - 0.01f, 0.0f, 1.0f, sd.og_nx);
	const int qx1 = obs_cell((q.x + r - sd.og_x0) * sd.og_inv + 0.01f, 0.0f, 1.0f, sd.og_nx);
	const int qy0 = obs_cell((q.y - r - sd.og_y0) * sd.og_inv - 0.01f, 0.0f, 1.0f, sd.og_ny);
	const int qy1 = obs_cell((q.y + r - sd.og_y0) * sd.og_inv + 0.01f, 0.0f, 1.0f, sd.og_ny);
	for (int cy = qy0; cy <= qy1; ++cy) {
		const int row = sd.og_start + cy * sd.og_nx;
		const int i0 = S.og_start[row + qx0], i1 = S.og_start[row + qx1 + 1];
		for (int b0 = i0; b0 < i1; b0 += 32) {
			const int it = b0 + lane;
			bool ok = false;
			int e = 0;
			if (it < i1) {
				const int2 item = S.og_items[it];
				e = item.x;
				const int4 ec = S.og_ecell[e];
				if (item.y == max(ec.x, qx0) && cy == max(ec.y, qy0)) {
					const float4 E = S.edges[e];
					ok = dist2_to_segment(q, V(E.x, E.y), V(E.z, E.w)) <= r2;
				}
			}
			const unsigned m = __ballot_sync(0xffffffffu, ok);
			if (ok) out[K + __popc(m & lt)] = (uint32_t)e;
			K += __popc(m);
		}
	}
	__syncwarp();
	// rank sort of the group's edge indices (distinct)
	const int cnt = K - gs;
	if (cnt <= 32) {
		const uint32_t v = lane < cnt ? out[gs + lane] : 0xffffffffu;
		int rank = 0;
		for (int j = 0; j < cnt; ++j) rank += __shfl_sync(0xffffffffu, v, j) < v;
		__syncwarp();
		if (lane < cnt) out[gs + rank] = ((uint32_t)g << 28) | v;
	} else {
		if (lane == 0) {
			for (int a = gs + 1; a < K; ++a) {
				const uint32_t v = out[a];
				int b = a - 1;
				while (b >= gs && out[b] > v) { out[b + 1] = out[b]; --b; }
				out[b + 1] = v;
			}
			for (int a = gs; a < K; ++a) out[a] |= (uint32_t)g << 28;
		}
	}
	__syncwarp();
	return K;
}

// Obstacle edges within range of the agent (worldBase.cpp:62-77), per
// displacement group as the agents (worldToric.cpp:32-79): edges in file
// order, each group's appended after the previous one.  Returns the count.
__device__ int gather_obstacles(const DevState& S, const ScenDesc& sd, float2 p, float r, int lane, uint32_t* out)
{
	int K = 0;
	const float r2 = r * r;
	const unsigned lt = (1u << lane) - 1u;
	for (int g = 0; g < 5; ++g) {
		float2 disp = V(0, 0);
		if (g > 0) {
			if (sd.world != W_TORIC) break;
			bool active;
			if (g == 1) { active = (p.x - r) < -0.5f * sd.width; disp = V(sd.width, 0); }
			else if (g == 2) { active = (p.x + r) > 0.5f * sd.width; disp = V(-sd.width, 0); }
			else if (g == 3) { active = (p.y - r) < -0.5f * sd.height; disp = V(0, sd.height); }
			else { active = (p.y + r) > 0.5f * sd.height; disp = V(0, -sd.height); }
			if (!active) continue;
		}
		const float2 q = vadd(p, disp);
		if (sd.og_nx == 0) {
			for (int b0 = 0; b0 < sd.nedges; b0 += 32) {
				const int k = b0 + lane;
				bool ok = false;
				if (k < sd.nedges) {
					const float4 E = S.edges[sd.edge_off + k];
					ok = dist2_to_segment(q, V(E.x, E.y), V(E.z, E.w)) <= r2;
				}
				const unsigned m = __ballot_sync(0xffffffffu, ok);
				if (ok) out[K + __popc(m & lt)] = ((uint32_t)g << 28) | (uint32_t)(sd.edge_off + k);
				K += __popc(m);
			}
			continue;
		}
		K = gather_obstacles_grid(S, sd, q, r, g, lane, out, K);
		__syncwarp();
	}
	__syncwarp();
	return K;
}

// ------------------------------------------------------------------------
// warp helpers
// ------------------------------------------------------------------------
// Adds f (this lane's term, used where `take` is set) to acc in lane order
// of the ballot, i.e. neighbour order.  All lanes end with the same acc.
__device__ __forceinline__ float2 ordered_accumulate(float2 acc, float2 f, bool take)
{
	unsigned m = __ballot_sync(0xffffffffu, take);
	while (m) {
		const int src = __ffs(m) - 1;
		const float fx = __shfl_sync(0xffffffffu, f.x, src);
		const float fy = __shfl_sync(0xffffffffu, f.y, src);
		acc.x += fx;
		acc.y += fy;
		m &= m - 1;
	}
	return acc;
}

// fx[0..K) summed by lane 0 and fy[0..K) by lane 1, in list order (the
// reference's sequential Vector2D sum), eight loads issued ahead of their
// additions; every lane returns both sums.
__device__ __forceinline__ float2 list_sum(const float* fx, const float* fy, int K, int lane)
{
	float acc = 0.0f;
	if (lane < 2) {
		const float* src = lane ? fy : fx;
		int k = 0;
		for (; k + 8 <= K; k += 8) {
			float v[8];
#pragma unroll
			for (int j = 0; j < 8; ++j) v[j] = src[k + j];
#pragma unroll
			for (int j = 0; j < 8; ++j) acc += v[j];
		}
		for (; k < K; ++k) acc += src[k];
	}
	return V(__shfl_sync(0xffffffffu, acc, 0), __shfl_sync(0xffffffffu, acc, 1));
}

__device__ float2 obstacle_force(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane);

// ObjectInteractionForces::ComputeForce: ObjectInteractionForces.cpp:26-48
// (agents only; obstacles add (0,0)); GoalReachingForce.cpp:26-29.
// Lanes evaluate one neighbour each into shared memory; lane 0 then adds the
// x terms and lane 1 the y terms in neighbour order, as the reference's
// sequential Vector2D sum does.
__device__ float2 compute_force(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane, float* fx, float* fy)
{
	if (c.kind == K_GOALREACHING) return vdiv(vsub(A.pref, A.vel), fmaxr(A.relax, A.dt));
	const float rs = c.range * c.range;
	if (c.kind == K_SOCIALFORCES) {
		const SfConst SK = sf_const(A, c);
		for (int k = lane; k < N.K; k += 32) {
			float2 f = V(0, 0);
			if (N.d2[k] <= rs) f = sf_force(A, SK, nb_pos(N, k), nb_E(N, k), nb_radius(N, k));
			fx[k] = f.x;
			fy[k] = f.y;
		}
	} else {
		for (int k = lane; k < N.K; k += 32) {
			float2 f = V(0, 0);
			if (N.d2[k] <= rs) f = pl_force(A, c, nb_pos(N, k), nb_vel(N, k), nb_radius(N, k));
			fx[k] = f.x;
			fy[k] = f.y;
		}
	}
	// neighbours beyond the cost's range hold +0.0 (see ordered_sums)
	__syncwarp();
	const float2 sum = list_sum(fx, fy, N.K, lane);
	__syncwarp();
	return vadd(sum, obstacle_force(A, N, c, lane));
}

// The obstacle edges within cost c's range, summed in list order
// (ObjectInteractionForces.cpp:40-45); PowerLaw has no obstacle force
// (PowerLaw.cpp:68-72: a zero vector each).
__device__ float2 obstacle_force(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane)
{
	const float rs = c.range * c.range;
	float2 obs = V(0, 0);
	if (c.kind == K_SOCIALFORCES) {
		for (int b0 = 0; b0 < N.KO; b0 += 32) {
			const int k = b0 + lane;
			bool take = false;
			float2 f = V(0, 0);
			if (k < N.KO) {
				float2 a, b;
				nb_seg(N, k, &a, &b);
				if (dist2_to_segment(A.pos, a, b) <= rs) { take = true; f = sf_obstacle_force(A, c, a, b); }
			}
			obs = ordered_accumulate(obs, f, take);
		}
	}
	return obs;
}

// ForceBasedFunction::ComputeTargetVelocity: ForceBasedFunction.cpp:48-52
__device__ __forceinline__ float2 target_velocity(const AgentCtx& A, const NbView& N, const CostDesc& c, int lane,
                                                  float* fx, float* fy)
{
	return vadd(A.vel, vmul(vdiv(compute_force(A, N, c, lane, fx, fy), c.p[5]), A.dt));
}

__device__ __forceinline__ bool is_force_based(int kind)
{
	return kind == K_SOCIALFORCES || kind == K_POWERLAW || kind == K_GOALREACHING;
}

// Solver::createAgentOrcaLines + solveOrcaProgram: ORCASolver.cpp:61-171
__device__ float2 orca_solve(const AgentCtx& A, const NbView& N, const CostDesc& c, float4* lines, float4* proj,
                             int* nlines_out, int lane)
{
	const float tH = c.p[0];
	const float maxDistSq = c.range * c.range;
	int nl = 0;
	for (int base = 0; base < N.K; base += 32) {
		const int k = base + lane;
		const bool in = k < N.K && N.d2[k] <= maxDistSq;
		float4 out = make_float4(0, 0, 0, 0);
		if (in) {
			const float2 relPos = vsub(nb_pos(N, k), A.pos);
			const float2 relVel = vsub(A.vel, nb_vel(N, k));
			const float distSq = vsq(relPos);
			const float cR = A.radius + nb_radius(N, k);
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
					const float dp2 = vdot(relVel, dir);
					u = vsub(vmul(dir, dp2), relVel);
				}
			} else {
				const float2 w = vsub(relVel, vdiv(relPos, A.dt));
				const float wLen = vsq(w);   // sic: ORCASolver.cpp:161
				const float2 unitW = vdiv(w, wLen);
				dir = V(unitW.y, -unitW.x);
				u = vmul(unitW, cR / A.dt - wLen);
			}
			const float2 pt = vadd(A.vel, vmul(u, 0.5f));
			out = make_float4(pt.x, pt.y, dir.x, dir.y);
		}
		const unsigned m = __ballot_sync(0xffffffffu, in);
		if (in) lines[nl + __popc(m & ((1u << lane) - 1u))] = out;
		nl += __popc(m);
	}
	__syncwarp();
	float2 res;
	const int fail = lp2(lines, nl, A.maxspeed, A.pref, false, &res, lane);
	if (fail < nl) lp3(lines, nl, fail, A.maxspeed, &res, proj, lane);
	*nlines_out = nl;
	return res;
}

// ------------------------------------------------------------------------
// gradients (uniform across the warp)
// ------------------------------------------------------------------------
// TtcaDca::GetGradient: TtcaDca.cpp:131-262
// Sums of per-neighbour terms in neighbour order: lane j < nsum adds z_j[0..K)
// sequentially (entries of neighbours that contribute nothing hold +0.0,
// which leaves a sum that starts at +0.0 unchanged: x + (+0) = x for x != -0,
// and such sums never reach -0.0).  Returns the sums in s[0..nsum).
__device__ __forceinline__ void ordered_sums(const float* z0, const float* z1, const float* z2, int nsum, int K,
                                             int lane, float* s)
{
	__syncwarp();
	float acc = 0.0f;
	if (lane < nsum) {
		const float* src = lane == 0 ? z0 : (lane == 1 ? z1 : z2);
		for (int k = 0; k < K; ++k) acc += src[k];
	}
	s[0] = __shfl_sync(0xffffffffu, acc, 0);
	s[1] = __shfl_sync(0xffffffffu, acc, 1);
	s[2] = __shfl_sync(0xffffffffu, acc, 2);
	__syncwarp();
}

// TtcaDca::GetGradient (TtcaDca.cpp:130-223): the per-neighbour terms
// lane-parallel into z0..z2, then the reference's three sums in order
__device__ float2 grad_ttcadca(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v, int lane, float* z0,
                               float* z1, float* z2)
{
	const float sA = c.p[0], sS = c.p[1], sT = c.p[2], sD = c.p[3];
	const float viewHalf = (float)(REF_PI / 2.0);
	const float eps = 0.001f;
	const float rs = c.range * c.range;
	for (int k = lane; k < N.K; k += 32) {
		z0[k] = 0.0f; z1[k] = 0.0f; z2[k] = 0.0f;
		if (N.d2[k] > rs) continue;
		const float2 np = nb_pos(N, k);
		const float nr = nb_radius(N, k);
		const float2 dpc = vsub(np, A.pos), dvc = vsub(nb_vel(N, k), v);
		if (angle_greater(dpc, A.vel, viewHalf, -4.3711388e-08f)) continue;
		const float dpMag = vmag(dpc);
		const float2 dp = vmul(vdiv(dpc, dpMag), dpMag - A.radius - nr);
		const float2 nrm = V(-dpc.y, dpc.x);
		const float2 dv = vadd(dvc, vmul(nrm, vdot(nrm, dvc)));
		const float dvSq = vsq(dv);
		float ttca = (dvSq == 0 ? 0 : -vdot(dp, dv) / dvSq);
		if (ttca < 0) ttca = 0;
		const float2 vdca = vadd(dp, vmul(dv, ttca));
		float dca = vmag(vdca);
		if (dca < 0) dca = 0;
		if (dvSq <= eps) continue;
		const float2 VelRot = V(dv.y, -dv.x);
		const float VelMag = sqrtf(dvSq);
		const float2 VelNorm = vdiv(dv, VelMag);
		float gTA = 0, gTS = 0;
		if (fabsf(ttca) > eps) {
			const float2 rel = vadd(dp, vmul(dv, 2 * ttca));
			gTA = -vdot(rel, VelRot) / dvSq;
			gTS = vdot(rel, VelNorm) / dvSq;
		}
		float gDA = 0, gDS = 0;
		if (fabsf(dca) > eps) {
			gDA = vdot(vdca, vadd(vmul(dv, gTA), vmul(VelRot, ttca))) / dca;
			gDS = vdot(vdca, vsub(vmul(dv, gTS), vmul(VelNorm, ttca))) / dca;
		}
		const float cost = ttcadca_pair_cost(ttca, dca, sT, sD);
		const float tf = ttca / (sT * sT), df = dca / (sD * sD);
		const float gCS = -cost * (gTS * tf + gDS * df);
		const float gCA = -cost * (gTA * tf + gDA * df);
		const float scale = 1 / vsq(dp);
		z0[k] = gCA * scale;
		z1[k] = gCS * scale;
		z2[k] = scale;
	}
	float sums[3];
	ordered_sums(z0, z1, z2, 3, N.K, lane, sums);
	float GradTh = sums[0], GradS = sums[1];
	const float total = sums[2];
	if (total > 0) { GradTh /= total; GradS /= total; }
	// getMovementCostGradient: TtcaDca.cpp:54-60 (counterClockwiseAngle)
	float alpha = vangle_exact(v, A.pref);
	if (vclockwise(v, A.pref)) alpha = -alpha;
	const float ds = vmag(v) - A.prefspeed;
	const double qa = (double)(alpha / sA), qs = (double)(ds / sS);
	const double DCa = __dmul_rn((double)(alpha / (2 * sA * sA)), exp(-0.5 * __dmul_rn(qa, qa)));
	const double DCs = __dmul_rn((double)(ds / (2 * sS * sS)), exp(-0.5 * __dmul_rn(qs, qs)));
	GradTh += (float)DCa;
	GradS += (float)DCs;
	if ((double)vsq(v) < 0.01)
		return rotate_gradient(GradTh, GradS, vnorm(A.pref), vmag(A.pref));
	return rotate_gradient(GradTh, GradS, vnorm(v), vmag(v));
}

// FOEAvoidance::GetGradient: FOEAvoidance.cpp:94-143
__device__ float2 grad_foe(const AgentCtx& A, const NbView& N, const CostDesc& c, float2 v, int lane, float* z0,
                           float* z1)
{
	if (viszero(v)) return V(0, 0);
	const float2 Vn = vnorm(v);
	const float rs = c.range * c.range;
	const double LN10 = 2.302585092994045684;
	for (int k = lane; k < N.K; k += 32) {
		z0[k] = 0.0f; z1[k] = 0.0f;
		if (N.d2[k] > rs) continue;
		const float2 dv = vsub(nb_vel(N, k), v), dp = vsub(nb_pos(N, k), A.pos);
		const float2 Vel = V(Vn.y * dv.x + -Vn.x * dv.y, Vn.x * dv.x + Vn.y * dv.y);
		const float2 Pos = V(Vn.y * dp.x + -Vn.x * dp.y, Vn.x * dp.x + Vn.y * dp.y);
		if (Pos.y < 0.1f || Vel.y >= -0.01f) continue;
		const float xf = Vel.x / Vel.y, xg = Pos.x / Pos.y, dx = xg - xf;
		const float ttc = -Pos.y / Vel.y;
		const float sigma = (float)__ddiv_rn((double)((A.radius + nb_radius(N, k)) / Pos.y), LN10);
		const float sg = (float)((0 < dx) - (dx < 0));
		const float E = foe_importance(ttc) * ref_expf(A.ex, -fabsf(dx) / sigma);
		z0[k] = E * sg * (xf * xf - xg * xg - (vmag(v) / (-Vel.y))) / sigma;
		z1[k] = E * sg * (-xf / (-Vel.y)) / sigma;
	}
	float sums[3];
	ordered_sums(z0, z1, z1, 2, N.K, lane, sums);
	float gt = sums[0];
	const float gv = sums[1];
	if (gt < -0.1f) gt = -0.1f;
	else if (gt > 0.1f) gt = 0.1f;
	float sn, cs;
	host_sincosf(gt, &sn, &cs);
	const float2 w = vadd(vmul(V(sn, 1 - cs), vmag(v)), V(0, gv));
	return V(-Vn.y * w.x + -Vn.x * w.y, -(-Vn.x) * w.x + -Vn.y * w.y);
}

}  // namespace umans
// cost-function plugins: their device functions may use the gradient
// helpers above (grad_foe, ordered_sums, ...)
#include "plugins.cuh"
namespace umans {

// ------------------------------------------------------------------------
// per-cost evaluation (sampling / finite differences)
// ------------------------------------------------------------------------
struct CostPrep {
	float2 target[MAX_COSTS];    // force-based target velocity
	float ttcp[MAX_COSTS];       // Karamouzas TTC at the preferred velocity
	float maxdev[MAX_COSTS], cosdev[MAX_COSTS];
	const float4* lines;         // ORCA lines
	int nlines;
	float2 orca_v;
};

__device__ float eval_cost(const AgentCtx& A, const NbView& N, const CostDesc& c, const CostPrep& P, int ci, float2 v)
{
	switch (c.kind) {
	case K_SOCIALFORCES: case K_POWERLAW: case K_GOALREACHING:
		return 0.5f * vsq(vsub(v, P.target[ci])) / A.dt;   // ForceBasedFunction.cpp:26-30
	case K_KARAMOUZAS: return cost_karamouzas(A, N, c, P.ttcp[ci], P.maxdev[ci], P.cosdev[ci], v);
	case K_MOUSSAID: return cost_moussaid(A, N, c, v);
	case K_VANTOLL: return cost_vantoll(A, N, c, v);
	case K_PLEDESTRIANS: return cost_pledestrians(A, N, c, v);
	case K_RVO: return cost_rvo(A, N, c, v);
	case K_ORCA: return cost_orca(A, P.lines, P.nlines, v);
	case K_PARIS: return cost_paris(A, N, c, v);
	case K_TTCADCA: return cost_ttcadca(A, N, c, v);
	case K_FOE: return cost_foe(A, N, c, v);
	case K_GENERIC: return 0;   // GenericCost::GetCost: GenericCost.cpp:27-31
	}
	if (c.kind >= K_PLUGIN0) return plugin_cost(c.kind - K_PLUGIN0, A, N, c, v);
	return 0;
}

__device__ __forceinline__ uint32_t mulmod(uint32_t a, uint32_t b)
{
	return (uint32_t)(((uint64_t)a * b) % LCG_M);
}
// generate_canonical<float,24> on minstd_rand0 state x, then a + u*(b-a)
__device__ __forceinline__ float rng_uniform(uint32_t x, float a, float b)
{
	const float sum = (float)(x - 1u);
	float ret = sum / 2147483648.0f;
	if (ret >= 1.0f) ret = 0.99999994f;   // nextafter(1, 0)
	return ret * (b - a) + a;
}

// CostFunction::ApproximateGlobalMinimumBySampling: costFunction.cpp:66-164.
// Samples are spread over lanes; the argmin keeps the first strict minimum.
// Samples of the Karamouzas window swept together (independent chains).
// Measured on a 100k-agent corridor (k_agent<3>, ms per step):
// 2: 17.9, 3: 17.3, 4: 16.8, 5: 17.1, 6: 17.2, 8: 20.5, 10: 23.5.
#ifndef UMANS_KS
#define UMANS_KS 4
#endif
constexpr int KS = UMANS_KS;

// KARA: every policy of the launch samples a regular schedule with one
// Karamouzas cost (the general sampler is compiled out)
template <bool KARA = false>
__device__ float2 sample_min(const DevState& S, const AgentCtx& A, const NbView& N, const PolicyDesc& pol,
                             const CostPrep& P, uint32_t rng0, int lane, float4* pair4, float* pairv)
{
	float2 base = V(0, 0);
	if (pol.table_base == 1) base = A.vel;
	float radius;
	if (pol.table_radius == 0) radius = A.prefspeed;
	else if (pol.table_radius == 1) radius = A.maxspeed;
	else radius = fminr(2.0f * A.maxspeed, A.maxacc * A.dt);
	float2 dir = V(1, 0);
	if (pol.table_dir == 1) dir = vnorm(A.vel);
	else if (pol.table_dir == 2) dir = vnorm(A.pref);
	const float dL = radius / (float)pol.len_divisor;
	const int ncost = pol.single_cost ? 1 : pol.ncost;
	float bestC = MAXF;
	int bestI = 0x7fffffff;
	if (KARA || (ncost == 1 && pol.cost[0].kind == K_KARAMOUZAS && !pol.table_random)) {
		// Karamouzas alone: most samples fall outside its window (cost MAXF);
		// the lanes test the windows of 32 samples at a time, then the warp
		// sweeps the neighbours for each sample inside, in sample order.
		const CostDesc& c = pol.cost[0];
		const float coeff = pol.single_cost ? 1.0f : c.coeff;
		const float outside = 0.0f + coeff * MAXF;   // the sum of one term, as below
		int first_out = 0x7fffffff;
		// the sample-invariant part of every pair within the cost's range,
		// compacted into this warp's scratch: ttc_pair's P = p - p_j and
		// c = |P|^2 - (r + r_j)^2 (c <= 0 exactly when |P|^2 <= (r + r_j)^2),
		// and the neighbour's velocity
		int KP = 0;
		{
			const float md2 = c.range * c.range;
			for (int b0 = 0; b0 < N.K; b0 += 32) {
				const int k = b0 + lane;
				const bool inr = k < N.K && !(N.d2[k] > md2);
				const unsigned m = __ballot_sync(0xffffffffu, inr);
				if (inr) {
					const float2 Pd = vsub(A.pos, nb_pos(N, k));
					const float R = A.radius + nb_radius(N, k);
					const float2 vj = nb_vel(N, k);
					const int idx = KP + __popc(m & ((1u << lane) - 1u));
					pair4[idx] = make_float4(Pd.x, Pd.y, vdot(Pd, Pd) - R * R, vj.x);
					pairv[idx] = vj.y;
				}
				KP += __popc(m);
			}
			__syncwarp();
		}
		unsigned long long n_in = 0;
		for (int i0 = 0; i0 < pol.nsamples; i0 += 32) {
			const int i = i0 + lane;
			float2 v = V(0, 0);
			float speed = 0;
			bool in = false, valid = i < pol.nsamples;
			if (valid) {
				const SampleEntry e = S.table[pol.table_offset + i];
				v = vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
				speed = vmag(v);
				in = karamouzas_window(A, P.ttcp[0], P.maxdev[0], P.cosdev[0], v, speed);
			}
			const unsigned out_mask = __ballot_sync(0xffffffffu, valid && !in);
			if (out_mask && first_out == 0x7fffffff) first_out = i0 + __ffs(out_mask) - 1;
			// KS samples inside the window at a time: their sweeps share the
			// pair loads and run as independent chains
			unsigned m = __ballot_sync(0xffffffffu, in);
			n_in += __popc(m);
			while (m) {
				int si[KS];
				float2 sv[KS];
				float ssp[KS], T[KS];
#pragma unroll
				for (int j = 0; j < KS; ++j) {
					si[j] = m ? __ffs(m) - 1 : -1;
					if (m) m &= m - 1;
					const int src = si[j] < 0 ? si[0] : si[j];
					sv[j] = V(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
					ssp[j] = __shfl_sync(0xffffffffu, speed, src);
					T[j] = MAXF;
				}
				// ComputeTimeToFirstCollision over the pairs (ignoring current
				// collisions): minima, split over the lanes
				for (int k = lane; k < KP; k += 32) {
					const float4 q = pair4[k];
					const float2 P2 = V(q.x, q.y), v2 = V(q.w, pairv[k]);
#pragma unroll
					for (int j = 0; j < KS; ++j) {
						const float t = ttc_pair_pre(sv[j], P2, q.z, v2);
						if (t != 0 && t < T[j]) T[j] = t;
					}
				}
				// obstacle edges within the cost's range
				for (int k = lane; k < N.KO; k += 32) {
					float2 a, b;
					nb_seg(N, k, &a, &b);
					if (dist2_to_segment(A.pos, a, b) > c.range * c.range) continue;
					for (int j = 0; j < KS; ++j) {
						const float t = ttc_segment(A.pos, sv[j], A.radius, a, b);
						if (t != 0 && t < T[j]) T[j] = t;
					}
				}
#pragma unroll
				for (int j = 0; j < KS; ++j)
					for (int o = 16; o > 0; o >>= 1) {
						const float x = __shfl_xor_sync(0xffffffffu, T[j], o);
						if (x < T[j]) T[j] = x;
					}
				// costs in sample order: the first strict minimum is kept
#pragma unroll
				for (int j = 0; j < KS; ++j) {
					if (si[j] < 0) break;
					const float tc = 0.0f + coeff * karamouzas_terms(A, c, sv[j], ssp[j], T[j]);
					if (tc < bestC) { bestC = tc; bestI = i0 + si[j]; }
				}
			}
		}
		if (S.counters && lane == 0) {
			atomicAdd(&S.counters[0], n_in);
			atomicAdd(&S.counters[1], n_in * (unsigned long long)KP);
			atomicAdd(&S.counters[2], 1ull);
		}
		// samples outside the window all cost `outside`; like every sample
		// they count only below the initial best (MAXF), and then the first
		// of them competes with the best inside on (cost, index)
		if (first_out != 0x7fffffff && outside < MAXF &&
		    (outside < bestC || (outside == bestC && first_out < bestI))) {
			bestC = outside;
			bestI = first_out;
		}
		if (bestI == 0x7fffffff) return V(0, 0);
		const SampleEntry e = S.table[pol.table_offset + bestI];
		return vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
	}
	// costs that take the time to first collision per sample: the
	// sample-invariant pair terms once per agent (not with ORCA, whose lines
	// use the same scratch)
	NbView NC = N;
	{
		float cr = -1.0f;
		bool orca = false;
		for (int ci = 0; ci < ncost; ++ci) {
			const int kd = pol.cost[ci].kind;
			orca |= kd == K_ORCA;
			if (cr < 0.0f && (kd == K_RVO || kd == K_VANTOLL || kd == K_PLEDESTRIANS || kd == K_MOUSSAID ||
			                  kd == K_KARAMOUZAS))
				cr = pol.cost[ci].range;
		}
		if (cr >= 0.0f && !orca) {
			const float md2 = cr * cr;
			int KP = 0;
			for (int b0 = 0; b0 < N.K; b0 += 32) {
				const int k = b0 + lane;
				const bool inr = k < N.K && !(N.d2[k] > md2);
				const unsigned m = __ballot_sync(0xffffffffu, inr);
				if (inr) {
					const float2 Pd = vsub(A.pos, nb_pos(N, k));
					const float R = A.radius + nb_radius(N, k);
					const float2 vj = nb_vel(N, k);
					const int idx = KP + __popc(m & ((1u << lane) - 1u));
					pair4[idx] = make_float4(Pd.x, Pd.y, vdot(Pd, Pd) - R * R, vj.x);
					pairv[idx] = vj.y;
				}
				KP += __popc(m);
			}
			__syncwarp();
			NC.pp = pair4;
			NC.pv = pairv;
			NC.KP = KP;
			NC.pp_range = cr;
		}
	}
	for (int i = lane; i < pol.nsamples; i += 32) {
		float2 v;
		const int d0 = i * pol.draws;   // draws before this sample
		if (pol.table_random) {
			const float ma = pol.max_angle;
			const uint32_t x1 = mulmod(S.lcgpow[d0 + 1], rng0);
			const uint32_t x2 = mulmod(S.lcgpow[d0 + 2], rng0);
			const float ra = rng_uniform(x1, -ma, ma);
			const float rl = rng_uniform(x2, 0, radius);
			float sn, cs;
			host_sincosf(ra, &sn, &cs);
			v = vadd(base, vmul(vrot_cs(dir, cs, sn), rl));
		} else {
			const SampleEntry e = S.table[pol.table_offset + i];
			v = vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
		}
		float tc = 0;
		int jr = d0 + (pol.table_random ? 2 : 0);
		for (int ci = 0; ci < ncost; ++ci) {
			const float coeff = pol.single_cost ? 1.0f : pol.cost[ci].coeff;
			float cv;
			if (pol.cost[ci].kind == K_RANDOM)   // RandomFunction::GetCost: RandomFunction.cpp:25-28
				cv = rng_uniform(mulmod(S.lcgpow[++jr], rng0), -1, 1);
			else
				cv = eval_cost(A, NC, pol.cost[ci], P, ci, v);
			tc += coeff * cv;
		}
		if (tc < bestC) { bestC = tc; bestI = i; }
	}
	for (int o = 16; o > 0; o >>= 1) {
		const float oc = __shfl_xor_sync(0xffffffffu, bestC, o);
		const int oi = __shfl_xor_sync(0xffffffffu, bestI, o);
		if (oc < bestC || (oc == bestC && oi < bestI)) { bestC = oc; bestI = oi; }
	}
	if (bestI == 0x7fffffff) return V(0, 0);
	// every lane rebuilds the winning candidate
	const int i = bestI;
	if (pol.table_random) {
		const float ma = pol.max_angle;
		const uint32_t x1 = mulmod(S.lcgpow[i * pol.draws + 1], rng0);
		const uint32_t x2 = mulmod(S.lcgpow[i * pol.draws + 2], rng0);
		const float ra = rng_uniform(x1, -ma, ma);
		const float rl = rng_uniform(x2, 0, radius);
		float sn, cs;
		host_sincosf(ra, &sn, &cs);
		return vadd(base, vmul(vrot_cs(dir, cs, sn), rl));
	}
	const SampleEntry e = S.table[pol.table_offset + i];
	return vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
}

// ------------------------------------------------------------------------
// the fused per-agent step
// ------------------------------------------------------------------------
// MODE 0: any policy.  MODE 1: every policy has force-based costs only
// (SocialForcesAvoidance, PowerLaw, GoalReachingForce), whatever its method
// (the velocity comes from the cost targets, finish_forces); the generic
// sampling, ORCA and finite-difference code is compiled out, which lowers
// register use and raises occupancy.
// TAPE: also record the neighbour lists and the pre-clamp acceleration for
// the differentiable form's backward pass
// OBST: the obstacle-edge gather compiled in (the force-only kernel of
// obstacle-free groups leaves it out, which keeps its registers)
// Agent::UpdateVelocityAndPosition (agent.cpp:71-93) for one agent: the
// contact force over the agent mass (80) added to the policy's velocity nv,
// the viewing direction, the new position (wrapped in toric worlds:
// worldToric.cpp:81-108).
__device__ __forceinline__ void update_agent(const DevState& S, const ScenDesc& sd, int slot, float2 pos,
                                             float2 pref, float dt, float2 nv, float2 contact)
{
	const float2 af = vdiv(contact, 80.0f);
	const float2 vel = vadd(nv, vmul(af, dt));
	const float2 vd = vdiv(vadd(vmul(vel, 2), pref), 3);
	// (double)|vd|^2 > 0.01 <=> |vd|^2 > 0.01f (0.01f is the float just below 0.01)
	if (vsq(vd) > 0.01f) S.view[slot] = vnorm(vd);
	float2 p = vadd(pos, vmul(vel, dt));
	if (sd.world == W_TORIC) {
		const float hw = 0.5f * sd.width, hh = 0.5f * sd.height;
		float x = p.x, y = p.y;
		if (x > hw) x -= sd.width;
		else if (x < -hw) x += sd.width;
		if (y > hh) y -= sd.height;
		else if (y < -hh) y += sd.height;
		p = V(x, y);
	}
	S.pos[slot] = p;
	S.vel[slot] = vel;
	S.vwf[slot] = nv;
}

// ------------------------------------------------------------------------
// agents to warps
// ------------------------------------------------------------------------
// Items [0, n) (agents, or groups of four agents) handed to the warps of a
// launch.  Schedule 0: warp w takes w, w + W, w + 2W, ... (W warps).
// Schedule 1: warp w a contiguous range.  Schedule 2, a work list: tiles of
// TILE items, each warp taking the next tile from the launch's counter
// when it has finished one; work_end then counts the warp out, and the last
// warp to finish resets the counter for the next launch (no warp waits).
struct WorkIter {
	int end, step;
};
// (WL false: the launch never uses the work list; its code is left out)
template <int TILE, bool WL>
__device__ __forceinline__ int work_take(const DevState& S, WorkIter& w, int lane, int n)
{
	unsigned k = 0;
	if (lane == 0) k = atomicAdd(S.work, 1u);
	k = __shfl_sync(0xffffffffu, k, 0);
	const long long b = (long long)k * TILE;
	if (b >= n) return -1;
	w.end = (int)min((long long)n, b + TILE);
	w.step = 1;
	return (int)b;
}
// the first item of the warp, the same on every lane; -1 when none
template <int TILE, bool WL = true>
__device__ __forceinline__ int work_first(const DevState& S, WorkIter& w, int n, int gw, int lane)
{
	if (WL && S.sched == 2) return work_take<TILE, WL>(S, w, lane, n);
	int i;
	if (S.sched == 1) {
		const int per = (n + S.total_warps - 1) / S.total_warps;
		i = gw * per; w.end = min(n, i + per); w.step = 1;
	} else { i = gw; w.end = n; w.step = S.total_warps; }
	return i < w.end ? i : -1;
}
// the item after i; -1 when none is left
template <int TILE, bool WL = true>
__device__ __forceinline__ int work_after(const DevState& S, WorkIter& w, int i, int lane, int n)
{
	i += w.step;
	if (i < w.end) return i;
	if (!WL || S.sched != 2) return -1;
	return work_take<TILE, WL>(S, w, lane, n);
}
template <bool WL = true>
__device__ __forceinline__ void work_end(const DevState& S, int lane)
{
	if (!WL || S.sched != 2 || lane != 0) return;
	const unsigned d = atomicAdd(S.work + 1, 1u);
	if (d == (unsigned)S.total_warps - 1u) {   // every warp has taken its last ticket
		S.work[0] = 0u;
		S.work[1] = 0u;
	}
}

// ------------------------------------------------------------------------
// force-only policies
// ------------------------------------------------------------------------
// Policies whose costs are all force-based (SocialForces, PowerLaw,
// GoalReaching), whatever their method, take this path.  Per agent the warp
// gathers the neighbour list and evaluates the neighbour terms: pair forces
// and contact forces in one pass over the list, each summed in list order.
// The per-agent remainder (GoalReachingForce, the cost targets and the
// method's choice of velocity, the clamps, Agent::UpdateVelocityAndPosition)
// then runs for up to 32 agents at once, one per lane, from a per-warp
// record in shared memory: t, the force of each cost (x, y), the contact
// force (x, y).  The stride is odd, so lane j's record starts in bank j.
constexpr int STASH_STRIDE = 2 + 2 * MAX_COSTS + 1;

// The neighbour force of cost c (SocialForces or PowerLaw; agents, then
// obstacle edges), as compute_force.  With contact_scale > 0 the same pass
// over the list also forms the agents' contact forces (policy.cpp:107-125)
// and sums them in list order into *contact.
__device__ float2 force_and_contact(const AgentCtx& A, const NbView& N, const CostDesc& c, float contact_scale,
                                    int lane, float* fx, float* fy, float2* contact)
{
	const float rs = c.range * c.range;
	const bool sf = c.kind == K_SOCIALFORCES;
	const SfConst SK = sf_const(A, c);
	float2 cacc = V(0, 0);
	for (int b0 = 0; b0 < N.K; b0 += 32) {
		const int k = b0 + lane;
		bool take = false;
		float2 fc = V(0, 0);
		if (k < N.K) {
			const float2 np = nb_pos(N, k);
			const float nr = nb_radius(N, k);
			const float d2 = N.d2[k];
			float2 f = V(0, 0);
			if (d2 <= rs) f = sf ? sf_force(A, SK, np, nb_E(N, k), nr) : pl_force(A, c, np, nb_vel(N, k), nr);
			fx[k] = f.x;
			fy[k] = f.y;
			if (contact_scale > 0) {
				// d2 is |pos - neighbour|^2 computed exactly as vsq(diff); if it
				// exceeds (r + r_j)^2 by 1e-5 relative, sqrt(d2) >= r + r_j and
				// the overlap test is false
				const float rsum = A.radius + nr;
				if (!(d2 > rsum * rsum * 1.00001f)) {
					const float2 diff = vsub(A.pos, np);
					const float inter = rsum - vmag(diff);
					if (inter > 0) { take = true; fc = vmul(vnorm(diff), contact_scale * inter); }
				}
			}
		}
		if (contact_scale > 0) cacc = ordered_accumulate(cacc, fc, take);
	}
	if (contact_scale > 0) *contact = cacc;
	__syncwarp();
	const float2 sum = list_sum(fx, fy, N.K, lane);
	__syncwarp();
	return vadd(sum, obstacle_force(A, N, c, lane));
}

// Karamouzas's per-agent terms (Karamouzas.cpp: the time to collision at the
// preferred velocity, its deviation window): the time is a min, so lanes
// split the neighbours.
__device__ __forceinline__ void karamouzas_prep(const AgentCtx& A, const NbView& N, const CostDesc& c, int ci,
                                                int lane, CostPrep* P)
{
	float m = MAXF;
	const float md2 = c.range * c.range;
	for (int k = lane; k < N.K; k += 32) {
		if (N.d2[k] > md2) continue;
		const float tt = ttc_pair(A.pos, A.pref, A.radius, nb_pos(N, k), nb_vel(N, k), nb_radius(N, k));
		if (tt == 0) continue;
		if (tt < m) m = tt;
	}
	for (int k = lane; k < N.KO; k += 32) {
		float2 a, b;
		nb_seg(N, k, &a, &b);
		if (dist2_to_segment(A.pos, a, b) > md2) continue;
		const float tt = ttc_segment(A.pos, A.pref, A.radius, a, b);
		if (tt == 0) continue;
		if (tt < m) m = tt;
	}
	for (int o = 16; o > 0; o >>= 1) {
		const float x = __shfl_xor_sync(0xffffffffu, m, o);
		if (x < m) m = x;
	}
	P->ttcp[ci] = m;
	P->maxdev[ci] = karamouzas_maxdev(m);
	P->cosdev[ci] = cosf(P->maxdev[ci]);
}

// Candidate velocity i of a sampling policy (costFunction.cpp:99-158): the
// regular schedule from its table, or random sampling with the agent's
// minstd_rand0 stream jumped ahead to the sample's draws.
__device__ __forceinline__ float2 sample_velocity(const DevState& S, const PolicyDesc& pol, float2 base, float2 dir,
                                                  float dL, float radius, uint32_t rng0, int i)
{
	if (pol.table_random) {
		const float ma = pol.max_angle;
		const uint32_t x1 = mulmod(S.lcgpow[i * pol.draws + 1], rng0);
		const uint32_t x2 = mulmod(S.lcgpow[i * pol.draws + 2], rng0);
		const float ra = rng_uniform(x1, -ma, ma);
		const float rl = rng_uniform(x2, 0, radius);
		float sn, cs;
		host_sincosf(ra, &sn, &cs);
		return vadd(base, vmul(vrot_cs(dir, cs, sn), rl));
	}
	const SampleEntry e = S.table[pol.table_offset + i];
	return vadd(base, vmul(vrot_cs(dir, e.c, e.s), dL * e.mult));
}

// The remainder of a batch of nb agents, lane j taking record j.  The
// policy's method picks the new velocity from the cost targets
// (ForceBasedFunction::ComputeTargetVelocity, ForceBasedFunction.cpp:48-52):
// - gradient: the gradient step of policy.cpp:78-89;
// - global with one cost: its target, the cost's global minimum
//   (ForceBasedFunction::GetGlobalMinimum);
// - sampling, or global with several costs (the default schedule of
//   SamplingParameters::ApproximateGlobalOptimization): the first sample of
//   least summed cost 0.5 |v - target|^2 / dt (ForceBasedFunction.cpp:26-30,
//   costFunction.cpp:60-95), one lane running the agent's samples in order.
// SAMP false: every policy of the group uses the gradient method (the
// other methods' code is compiled out).
template <bool TAPE, bool SAMP>
__device__ void finish_forces(const DevState& S, const float* stash, int nb, int lane)
{
	if (lane >= nb) return;
	const float* rec = stash + lane * STASH_STRIDE;
	const int t = __float_as_int(rec[0]);
	const int slot = S.sSlot[t];
	const float4 sb = S.sB[t];
	const float4 prm = S.prm[slot];
	const PolicyDesc& pol = S.pols[S.pol[slot]];
	const ScenDesc& sd = S.scen[S.agent_scen[slot]];
	const float2 pos = S.sP[t], vel = S.sV[t], pref = V(sb.x, sb.y);
	const float dt = sd.dt;
	float2 nv = V(0, 0);
	if (!viszero(pref)) {
		float2 acc;
		if (!SAMP || pol.method == M_GRADIENT) {
			float2 T = V(0, 0);
			for (int ci = 0; ci < pol.ncost; ++ci) {
				const CostDesc& c = pol.cost[ci];
				const float2 F = c.kind == K_GOALREACHING ? vdiv(vsub(pref, vel), fmaxr(pol.relax_time, dt))
				                                          : V(rec[1 + 2 * ci], rec[2 + 2 * ci]);
				const float2 target = vadd(vel, vmul(vdiv(F, c.p[5]), dt));
				T = vadd(T, vmul(vdiv(vsub(vel, target), dt), c.coeff));
			}
			acc = vmul(T, -1);
			if (TAPE) S.tape_acc[slot] = acc;
		} else {
			float2 tg[MAX_COSTS];
#pragma unroll
			for (int ci = 0; ci < MAX_COSTS; ++ci) {
				if (ci >= pol.ncost) break;
				const CostDesc& c = pol.cost[ci];
				const float2 F = c.kind == K_GOALREACHING ? vdiv(vsub(pref, vel), fmaxr(pol.relax_time, dt))
				                                          : V(rec[1 + 2 * ci], rec[2 + 2 * ci]);
				tg[ci] = vadd(vel, vmul(vdiv(F, c.p[5]), dt));
			}
			float2 best = V(0, 0);
			if (!pol.use_sampling) {
				best = tg[0];
			} else {
				// sample_min's schedule (base, direction, length step)
				float2 base = V(0, 0);
				if (pol.table_base == 1) base = vel;
				float radius;
				if (pol.table_radius == 0) radius = prm.y;
				else if (pol.table_radius == 1) radius = prm.z;
				else radius = fminr(2.0f * prm.z, prm.w * dt);
				float2 dir = V(1, 0);
				if (pol.table_dir == 1) dir = vnorm(vel);
				else if (pol.table_dir == 2) dir = vnorm(pref);
				const float dL = radius / (float)pol.len_divisor;
				const uint32_t r0 = S.rng[slot];
				float bestC = MAXF;
				int bestI = -1;
				for (int i = 0; i < pol.nsamples; ++i) {
					const float2 v = sample_velocity(S, pol, base, dir, dL, radius, r0, i);
					float tc = 0;
#pragma unroll
					for (int ci = 0; ci < MAX_COSTS; ++ci) {
						if (ci >= pol.ncost) break;
						tc += pol.cost[ci].coeff * (0.5f * vsq(vsub(v, tg[ci])) / dt);
					}
					if (tc < bestC) { bestC = tc; bestI = i; }
				}
				if (bestI >= 0) best = sample_velocity(S, pol, base, dir, dL, radius, r0, bestI);
				if (pol.draws > 0) S.rng[slot] = mulmod(S.lcgpow[pol.nsamples * pol.draws], r0);
			}
			acc = vdiv(vsub(best, vel), fmaxr(pol.relax_time, dt));
		}
		acc = vclamp(acc, prm.w);
		nv = vclamp(vadd(vel, vmul(acc, dt)), prm.z);
	}
	update_agent(S, sd, slot, pos, pref, dt, nv, V(rec[2 * MAX_COSTS + 1], rec[2 * MAX_COSTS + 2]));
}

template <bool TAPE, bool OBST, bool SAMP>
__device__ void force_agents(const DevState& S, const WarpLists& L, float* stash, int lane, int gw, bool* overflow)
{
	float* fx = reinterpret_cast<float*>(L.nid);
	float* fy = L.aux;
	WorkIter w;
	const int n_items = S.t_end - S.t_begin;
	int nb = 0;
	for (int it = work_first<32>(S, w, n_items, gw, lane); it >= 0; it = work_after<32>(S, w, it, lane, n_items)) {
		const int t = S.t_begin + it;
		const int slot = S.sSlot[t];
		const float4 sb = S.sB[t];
		const float4 prm = S.prm[slot];
		const PolicyDesc& pol = S.pols[S.pol[slot]];
		AgentCtx A;
		A.pos = S.sP[t]; A.vel = S.sV[t]; A.pref = V(sb.x, sb.y); A.goal = V(0, 0);
		A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
		const int sc = S.agent_scen[slot];
		const ScenDesc sd = S.scen[sc];
		const GridParams G = S.grid[sc];
		A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;

		const int K = gather(S, G, S.cell_base[sc], sd.world, sd.width, sd.height, L, t, A.pos, pol.range, lane, overflow);
		NbView N;
		N.ref = L.ref; N.d2 = L.key; N.K = K; N.sP = S.sP; N.sV = S.sV; N.sB = S.sB; N.sE = S.sE;
		N.W = sd.width; N.H = sd.height;
		N.edges = S.edges; N.obs = nullptr; N.KO = 0;
		if (TAPE) {
			for (int k = lane; k < K; k += 32) {
				const uint32_t rr = L.ref[k];
				S.tape_list[(size_t)slot * S.maxnb + k] = (rr & 0xF0000000u) | (uint32_t)S.sSlot[rr & 0x0FFFFFFFu];
			}
			if (lane == 0) S.tape_cnt[slot] = K;
		}
		if (OBST && sd.nedges > 0) {
			uint32_t* ol = S.obs_list + (size_t)gw * S.max_obs;
			N.KO = gather_obstacles(S, sd, A.pos, pol.range, lane, ol);
			N.obs = ol;
		}

		float* rec = stash + nb * STASH_STRIDE;
		float2 contact = V(0, 0);
		bool contact_done = !(pol.contact_scale > 0);
		if (!viszero(A.pref)) {
			for (int ci = 0; ci < pol.ncost; ++ci) {
				const CostDesc& c = pol.cost[ci];
				if (c.kind == K_GOALREACHING) continue;
				const float2 f = force_and_contact(A, N, c, contact_done ? 0.0f : pol.contact_scale, lane, fx, fy,
				                                   &contact);
				contact_done = true;
				if (lane == 0) { rec[1 + 2 * ci] = f.x; rec[2 + 2 * ci] = f.y; }
			}
		}
		// contact forces (policy.cpp:107-141): the agents, when no cost pass
		// formed them, then the colliding obstacle edges
		if (!contact_done) {
			for (int b0 = 0; b0 < K; b0 += 32) {
				const int k = b0 + lane;
				bool take = false;
				float2 f = V(0, 0);
				if (k < K) {
					const float rsum = A.radius + nb_radius(N, k);
					if (!(N.d2[k] > rsum * rsum * 1.00001f)) {
						const float2 diff = vsub(A.pos, nb_pos(N, k));
						const float inter = rsum - vmag(diff);
						if (inter > 0) { take = true; f = vmul(vnorm(diff), pol.contact_scale * inter); }
					}
				}
				contact = ordered_accumulate(contact, f, take);
			}
		}
		if (OBST && pol.contact_scale > 0) {
			for (int b0 = 0; b0 < N.KO; b0 += 32) {
				const int k = b0 + lane;
				bool take = false;
				float2 f = V(0, 0);
				if (k < N.KO) {
					float2 a, b;
					nb_seg(N, k, &a, &b);
					const float2 diff = vsub(A.pos, nearest_on_segment(A.pos, a, b));
					const float inter = A.radius - vmag(diff);
					if (inter > 0) { take = true; f = vmul(vnorm(diff), pol.contact_scale * inter); }
				}
				contact = ordered_accumulate(contact, f, take);
			}
		}
		if (lane == 0) {
			rec[0] = __int_as_float(t);
			rec[2 * MAX_COSTS + 1] = contact.x;
			rec[2 * MAX_COSTS + 2] = contact.y;
		}
		if (++nb == 32) {
			__syncwarp();
			finish_forces<TAPE, SAMP>(S, stash, nb, lane);
			__syncwarp();
			nb = 0;
		}
	}
	if (nb > 0) {
		__syncwarp();
		finish_forces<TAPE, SAMP>(S, stash, nb, lane);
	}
	work_end(S, lane);
}

// ------------------------------------------------------------------------
// force-only policies, four agents per warp
// ------------------------------------------------------------------------
// force_agents with eight lanes per agent: four agents per warp, consecutive
// in cell order (so that their lists have similar lengths).  Every loop runs
// warp-uniformly to the largest of the four agents' trip counts, each
// agent's lanes predicated on their own; shuffles stay within an agent's
// eight lanes (width 8) and each agent takes its byte of a ballot.  An
// agent's list is two arrays in shared memory (reference, key); the force
// pass overwrites each entry in place with its force terms (x over the key,
// y over the reference).  Worlds without obstacle edges whose policies have
// at most one neighbour cost (SocialForces or PowerLaw) take this path.
constexpr int QG = 8, QN = 32 / QG;

struct QLane {
	int sg, sl;        // agent of this lane in the warp, lane within the agent
	int shift;         // QG * sg
	unsigned below;    // the agent's lanes below this one
};
__device__ __forceinline__ unsigned q_ballot(bool p, const QLane& q)
{
	return (__ballot_sync(0xffffffffu, p) >> q.shift) & 0xFFu;
}
template <class T>
__device__ __forceinline__ T q_shfl(T v, int src) { return __shfl_sync(0xffffffffu, v, src, QG); }
__device__ __forceinline__ int q_max(int v) { return __reduce_max_sync(0xffffffffu, v); }

// warp_sort_regs for a group of G lanes (sl: the lane in the group): P = G M
// <= 64 packed keys, M per lane; entry i = G m + sl.  Exchanges at distances
// of G and more are between a lane's own registers.  The sorted keys also
// give the near-tie flags of fix_near_ties (pair (i, i+1) within the relative
// window win): every lane of the group returns the first and last flagged
// pair in *f0, *f1 (*f0 > *f1 when none is flagged).
template <int G, int M>
__device__ __forceinline__ void group_sort_regs(const WarpLists& L, int s, int len, int sl, float win, int* f0,
                                                int* f1)
{
	constexpr int QG = G;
	struct { int sl; } q{ sl };
	constexpr int P = QG * M;
	static_assert(P <= 64, "positions take at most 6 bits");
	constexpr int PB = P <= 32 ? 5 : 6;
	constexpr uint32_t PMASK = (1u << PB) - 1u;
	uint32_t u[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		u[m] = (i < len) ? ((__float_as_uint(L.key[s + i]) & ~PMASK) | (uint32_t)i) : 0xffffffffu;
	}
#pragma unroll
	for (int size = 2; size <= P; size <<= 1) {
#pragma unroll
		for (int j = size >> 1; j > 0; j >>= 1) {
#pragma unroll
			for (int m = 0; m < M; ++m) {
				const int i = m * QG + q.sl;
				const bool up = (i & size) == 0;
				if (j >= QG) {
					const int mm = m ^ (j / QG);
					if (mm > m) {
						const uint32_t a = u[m], b = u[mm];
						if (up ? (a > b) : (a < b)) { u[m] = b; u[mm] = a; }
					}
				} else {
					const uint32_t o = __shfl_xor_sync(0xffffffffu, u[m], j, QG);
					const bool lower = (q.sl & j) == 0;
					u[m] = (lower == up) ? min(u[m], o) : max(u[m], o);
				}
			}
		}
	}
	float k[M];
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		const int from = s + (int)(u[m] & PMASK);
		k[m] = (i < len) ? L.key[from] : 0.0f;
		u[m] = (i < len) ? L.ref[from] : 0u;
	}
	__syncwarp();
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		if (i < len) {
			L.ref[s + i] = u[m];
			L.key[s + i] = k[m];
		}
	}
	int lo = 0x7fffffff, hi = -1;
#pragma unroll
	for (int m = 0; m < M; ++m) {
		const int i = m * QG + q.sl;
		// the key of entry i + 1: the next lane's, or lane 0's next register
		const float a = __shfl_down_sync(0xffffffffu, k[m], 1, QG);
		const float b = __shfl_sync(0xffffffffu, k[m + 1 < M ? m + 1 : m], 0, QG);
		const float nx = q.sl < QG - 1 ? a : b;
		if (i + 1 < len && nx - k[m] <= win * nx) { lo = min(lo, i); hi = max(hi, i); }
	}
#pragma unroll
	for (int o = 1; o < QG; o <<= 1) {
		lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o, QG));
		hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o, QG));
	}
	*f0 = lo;
	*f1 = hi;
	__syncwarp();
}

// warp_sort (bitonic in shared memory, by (key, id)) for an agent's eight
// lanes; the network is sized for the longest of the four lists.
__device__ void q_sort_smem(const DevState& S, const WarpLists& L, int s, int len, int netlen, const QLane& q)
{
	if (netlen <= 1) return;
	int lp = 0;
	while ((1 << lp) < netlen) ++lp;
	const int halfP = 1 << (lp - 1);
	for (int ls = 1; ls <= lp; ++ls) {
		const int lh = ls - 1;
		for (int k = q.sl; k < halfP; k += QG) {
			const int blk = k >> lh, pos = k & ((1 << lh) - 1);
			const int lo = (blk << ls) + pos, hi = (blk << ls) + (1 << ls) - 1 - pos;
			if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
		}
		__syncwarp();
		for (int lj = lh - 1; lj >= 0; --lj) {
			for (int k = q.sl; k < halfP; k += QG) {
				const int lo = ((k >> lj) << (lj + 1)) | (k & ((1 << lj) - 1)), hi = lo + (1 << lj);
				if (hi < len) nb_cmpswap(S, L, s + lo, s + hi);
			}
			__syncwarp();
		}
	}
}

// The first and last pair (i, i+1) of the agent's sorted list [s, e) whose
// keys are within the relative window win (as fix_near_ties; *f0 > *f1 when
// none), on every lane of the agent.
__device__ void q_near_ties(const WarpLists& L, int s, int e, const QLane& q, float win, int* f0, int* f1)
{
	const int npairs = e - 1 - s;
	const int pmax = q_max(npairs);
	int lo = 0x7fffffff, hi = -1;
	for (int b = 0; b < pmax; b += QG) {
		const int i = b + q.sl;
		if (i < npairs) {
			const float a = L.key[s + i], c = L.key[s + i + 1];
			if (c - a <= win * c) { lo = min(lo, i); hi = max(hi, i); }
		}
	}
#pragma unroll
	for (int o = 1; o < QG; o <<= 1) {
		lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o, QG));
		hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o, QG));
	}
	*f0 = lo;
	*f1 = hi;
}

// fix_near_ties for an agent's eight lanes, given its first and last flagged
// pairs f0 <= f1 (relative to s): the agent's first lane walks the pairs
// between them and re-sorts each run of near-equal keys in the reference's
// order (runs are disjoint, and re-sorting one changes no flag of the pairs
// after it).
__device__ void q_fix_near_ties(const DevState& S, const WarpLists& L, int s, int f0, int f1, float2 qp,
                                const QLane& q, float win)
{
	if (!__any_sync(0xffffffffu, f0 <= f1)) return;
	__syncwarp();
	if (f0 <= f1 && q.sl == 0) {
		int k = s + f0;
		const int kend = s + f1;   // the last flagged pair
		while (k <= kend) {
			const float a = L.key[k], c = L.key[k + 1];
			if (c - a <= win * c) {
				const int r0 = k;
				++k;
				while (k <= kend) {
					const float a2 = L.key[k], c2 = L.key[k + 1];
					if (!(c2 - a2 <= win * c2)) break;
					++k;
				}
				sort_run(S, L, r0, k, qp);   // pairs r0 .. k-1 flagged: entries r0 .. k
			}
			++k;
		}
	}
	__syncwarp();
}

// gather for an agent's eight lanes (live false: an empty list).
__device__ int q_gather(const DevState& S, const GridParams& G, int cb, int world, float W, float H,
                        const WarpLists& L, int t, float2 p, float r, bool live, const QLane& q, bool* overflow)
{
	int K = 0, K0 = 0;
	const int maxnb = S.maxnb;
	live = live && r > 0;   // dist < r*r never holds for r = 0
	const float r2 = r * r;
	const double r2d = (double)r2;
	const float r2lo = r2 * 0.999999f, r2hi = r2 * 1.000001f;
	for (int g = 0; g < 5; ++g) {
		float2 disp = V(0, 0);
		bool active = live;
		if (g > 0) {
			// worldToric.cpp:64-76 (see gather)
			if (world != W_TORIC) active = false;
			else if (g == 1) { active = active && (p.x - r) < -0.5f * W; disp = V(W, 0); }
			else if (g == 2) { active = active && (p.x + r) > 0.5f * W; disp = V(-W, 0); }
			else if (g == 3) { active = active && (p.y - r) < -0.5f * H; disp = V(0, H); }
			else { active = active && (p.y + r) > 0.5f * H; disp = V(0, -H); }
		}
		if (__any_sync(0xffffffffu, active)) {
			const float2 qp = vadd(p, disp);
			const int gs = K;
			int cx0 = 0, cx1 = -1, cy0 = 0, nrows = 0;
			if (active) {
				cx0 = cell_coord((qp.x - r - G.x0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.nx);
				cx1 = cell_coord((qp.x + r - G.x0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.nx);
				cy0 = cell_coord((qp.y - r - G.y0) * G.inv_cs - 0.01f, 0.0f, 1.0f, G.ny);
				const int cy1 = cell_coord((qp.y + r - G.y0) * G.inv_cs + 0.01f, 0.0f, 1.0f, G.ny);
				nrows = cy1 - cy0 + 1;
			}
			const int maxrows = q_max(nrows);
			// QG rows at a time: lane k loads the sorted range of row k, the rows
			// are concatenated and scanned two chunks of QG candidates per pass
			for (int r0 = 0; r0 < maxrows; r0 += QG) {
				const int nr = nrows - r0;
				int rs = 0, len = 0;
				if (q.sl < nr) {
					const int c0 = cb + (cy0 + r0 + q.sl) * G.nx;
					rs = S.start[c0 + cx0];
					len = S.start[c0 + cx1 + 1] - rs;
				}
				int incl = len;
#pragma unroll
				for (int o = 1; o < QG; o <<= 1) {
					const int v = __shfl_up_sync(0xffffffffu, incl, o, QG);
					if (q.sl >= o) incl += v;
				}
				const int beg = incl - len;
				const int total = q_shfl(incl, QG - 1);
				const int maxtotal = q_max(total);
				for (int base = 0; base < maxtotal; base += 2 * QG) {
					const int nh = base + QG < maxtotal ? 2 : 1;
					int tt[2];
					float2 cp[2];
#pragma unroll
					for (int h = 0; h < 2; ++h) {
						if (h >= nh) break;
						const int c = base + QG * h + q.sl;
						int rr = 0;
#pragma unroll
						for (int step = QG / 2; step > 0; step >>= 1)
							if (q_shfl(beg, rr + step) <= c) rr += step;
						tt[h] = q_shfl(rs, rr) + (c - q_shfl(beg, rr));
						cp[h] = (c < total && tt[h] != t) ? S.sP[tt[h]] : V(0, 0);
					}
#pragma unroll
					for (int h = 0; h < 2; ++h) {
						if (h >= nh) break;
						const int c = base + QG * h + q.sl;
						bool ok = false;
						float d2f = 0;
						if (c < total && tt[h] != t) {
							const float dx = qp.x - cp[h].x, dy = qp.y - cp[h].y;
							d2f = dx * dx + dy * dy;
							if (d2f < r2lo) ok = true;
							else if (d2f <= r2hi) ok = exact_key(qp, cp[h]) < r2d;
						}
						const unsigned m = q_ballot(ok, q);
						if (ok) {
							const int idx = K + __popc(m & q.below);
							if (idx < maxnb) {
								L.ref[idx] = ((uint32_t)g << 28) | (uint32_t)tt[h];
								L.key[idx] = d2f;
							}
						}
						K += __popc(m);
					}
				}
			}
			if (K > maxnb) { *overflow = true; K = maxnb; }
			__syncwarp();
			// one register network (64 entries: a single instantiation keeps
			// the kernel's code small), the shared-memory sort beyond it
			const int len = K - gs;
			const int lmax = q_max(len);
			const float win = lmax <= 64 ? 0x1p-16f : 1e-6f;
			int f0, f1;
			if (lmax <= 64) {
				group_sort_regs<QG, 8>(L, gs, len, q.sl, win, &f0, &f1);
			} else {
				q_sort_smem(S, L, gs, len, lmax, q);
				q_near_ties(L, gs, K, q, win, &f0, &f1);
			}
			q_fix_near_ties(S, L, gs, f0, f1, qp, q, win);
		}
		if (g == 0) K0 = K;
	}
	// PhantomAgent::distSqr of the displaced entries (see gather)
	const int dmax = q_max(K - K0);
	for (int b = 0; b < dmax; b += QG) {
		const int k = K0 + b + q.sl;
		if (k < K) {
			const uint32_t rr = L.ref[k];
			const float2 ph = vadd(S.sP[rr & 0x0FFFFFFFu], group_offset(rr >> 28, W, H));
			L.key[k] = vsq(vsub(p, ph));
		}
	}
	__syncwarp();
	return K;
}

// force_and_contact for an agent's eight lanes, writing the force terms in
// place.  c: the agent's neighbour cost (null: none, or a zero preferred
// velocity); contact_scale 0: no contact forces.  Returns the cost's force
// (agents, then the (0, 0) of the absent obstacles), on all of the agent's
// lanes.
// SF: every neighbour cost of the launch is SocialForces (PowerLaw's code left out)
template <bool SF = false>
__device__ float2 q_force(const DevState& S, const AgentCtx& A, const WarpLists& L, int K, const CostDesc* c,
                          float contact_scale, float W, float H, const QLane& q, float2* contact)
{
	const float rs = c ? c->range * c->range : -1.0f;
	const bool sf = SF || (c && c->kind == K_SOCIALFORCES);
	SfConst SK = {};
	if (c) SK = sf_const(A, *c);
	float2 cacc = V(0, 0);
	const int kmax = q_max(K);
	for (int b0 = 0; b0 < kmax; b0 += QG) {
		const int k = b0 + q.sl;
		bool take = false;
		float2 fc = V(0, 0);
		if (k < K) {
			const uint32_t rr = L.ref[k];
			const int j = (int)(rr & 0x0FFFFFFFu);
			const float2 np = vadd(S.sP[j], group_offset(rr >> 28, W, H));
			const float4 E = S.sE[j];   // (normalised preferred velocity, speed, radius)
			const float nr = E.w;
			const float d2 = L.key[k];
			float2 f = V(0, 0);
			if (d2 <= rs) {
				if (SF || sf) f = sf_force(A, SK, np, E, nr);
				else if constexpr (!SF) f = pl_force(A, *c, np, S.sV[j], nr);
			}
			L.key[k] = f.x;
			L.ref[k] = __float_as_uint(f.y);
			if (contact_scale > 0) {
				// policy.cpp:107-125 (see force_and_contact)
				const float rsum = A.radius + nr;
				if (!(d2 > rsum * rsum * 1.00001f)) {
					const float2 diff = vsub(A.pos, np);
					const float inter = rsum - vmag(diff);
					if (inter > 0) { take = true; fc = vmul(vnorm(diff), contact_scale * inter); }
				}
			}
		}
		// contact terms added in list order
		unsigned m = q_ballot(take, q);
		while (__any_sync(0xffffffffu, m != 0u)) {
			const int src = m ? __ffs(m) - 1 : 0;
			const float fx = q_shfl(fc.x, src), fy = q_shfl(fc.y, src);
			if (m) {
				cacc.x += fx;
				cacc.y += fy;
				m &= m - 1;
			}
		}
	}
	*contact = cacc;
	__syncwarp();
	// the sums in list order: lane 0 the x terms, lane 1 the y terms
	float acc = 0.0f;
	if (c && q.sl < 2) {
		const uint32_t* src = q.sl ? L.ref : reinterpret_cast<const uint32_t*>(L.key);
		int k = 0;
		for (; k + 8 <= K; k += 8) {
			float v[8];
#pragma unroll
			for (int jj = 0; jj < 8; ++jj) v[jj] = __uint_as_float(src[k + jj]);
#pragma unroll
			for (int jj = 0; jj < 8; ++jj) acc += v[jj];
		}
		for (; k < K; ++k) acc += __uint_as_float(src[k]);
	}
	const float2 sum = V(q_shfl(acc, 0), q_shfl(acc, 1));
	__syncwarp();
	return vadd(sum, V(0, 0));
}

constexpr int QPAD = 8;
__host__ __device__ constexpr size_t q_words(int maxnb) { return 2 * (size_t)maxnb + QPAD; }

// One group of four agents (qi: its index in the launch's range) of
// k_force_quad: the gather, the force pass, the agents' records; every 32
// records, the per-agent remainder.
template <bool TAPE, bool SAMP, bool SF>
__device__ __forceinline__ void quad_step(const DevState& S, const QLane& q, const WarpLists& L, float* stash,
                                          int lane, int qi, int& nb, bool& overflow)
{
	const int maxnb = S.maxnb;
	const int t = S.t_begin + qi * QN + q.sg;
	const bool valid = t < S.t_end;
	const int tc = valid ? t : S.t_end - 1;   // in-range loads for a missing fourth agent
	const int slot = S.sSlot[tc];
	const float4 sb = S.sB[tc];
	const float4 prm = S.prm[slot];
	const PolicyDesc& pol = S.pols[S.pol[slot]];
	AgentCtx A;
	A.pos = S.sP[tc]; A.vel = S.sV[tc]; A.pref = V(sb.x, sb.y); A.goal = V(0, 0);
	A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
	const int sc = S.agent_scen[slot];
	const ScenDesc& sd = S.scen[sc];
	const GridParams G = S.grid[sc];
	A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;
	const float W = sd.width, H = sd.height;

	const int K = q_gather(S, G, S.cell_base[sc], sd.world, W, H, L, t, A.pos, pol.range, valid, q, &overflow);
	if (TAPE) {
		const int kmax = q_max(K);
		for (int b = 0; b < kmax; b += QG) {
			const int k = b + q.sl;
			if (k < K) {
				const uint32_t rr = L.ref[k];
				S.tape_list[(size_t)slot * maxnb + k] = (rr & 0xF0000000u) | (uint32_t)S.sSlot[rr & 0x0FFFFFFFu];
			}
		}
		if (valid && q.sl == 0) S.tape_cnt[slot] = K;
		__syncwarp();
	}
	int ci = -1;
	for (int k = 0; k < pol.ncost; ++k)
		if (pol.cost[k].kind != K_GOALREACHING) ci = k;
	const CostDesc* cd = (valid && ci >= 0 && !viszero(A.pref)) ? &pol.cost[ci] : nullptr;
	float2 contact;
	const float2 f = q_force<SF>(S, A, L, K, cd, valid ? pol.contact_scale : 0.0f, W, H, q, &contact);
	if (valid && q.sl == 0) {
		float* rec = stash + (nb + q.sg) * STASH_STRIDE;
		rec[0] = __int_as_float(t);
		if (ci >= 0) { rec[1 + 2 * ci] = f.x; rec[2 + 2 * ci] = f.y; }
		rec[2 * MAX_COSTS + 1] = contact.x;
		rec[2 * MAX_COSTS + 2] = contact.y;
	}
	nb += __popc(__ballot_sync(0xffffffffu, valid && q.sl == 0));
	if (nb > 32 - QN) {
		__syncwarp();
		finish_forces<TAPE, SAMP>(S, stash, nb, lane);
		__syncwarp();
		nb = 0;
	}
}

// WL: compiled for the work-list schedule (schedule 2), which it then
// requires; the other schedules use the variant without it.  SF: every
// neighbour cost of the group is SocialForces.
template <bool TAPE, bool SAMP = false, bool WL = false, bool SF = false>
__global__ void __launch_bounds__(128, 8) k_force_quad(DevState S)
{
	extern __shared__ unsigned char smem[];
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
	QLane q;
	q.sg = lane / QG; q.sl = lane % QG; q.shift = QG * q.sg; q.below = (1u << q.sl) - 1u;
	const int maxnb = S.maxnb;
	// an agent's arrays start QPAD words (8 banks) after the previous agent's
	// and its keys QPAD / 2 words after its references, so that the four
	// agents' lanes, and an agent's two summing lanes, fall in distinct banks
	uint32_t* lists = reinterpret_cast<uint32_t*>(smem) + ((size_t)wib * QN + q.sg) * q_words(maxnb);
	const WarpLists L{ lists, reinterpret_cast<float*>(lists + maxnb + QPAD / 2), nullptr, nullptr };
	float* stash = reinterpret_cast<float*>(smem) + (size_t)(blockDim.x >> 5) * QN * q_words(maxnb) + wib * 32 * STASH_STRIDE;
	bool overflow = false;
	const int nq = (S.t_end - S.t_begin + QN - 1) / QN;
	int nb = 0;
	if constexpr (WL) {
		WorkIter w;
		for (int qi = work_first<32 / QN>(S, w, nq, gw, lane); qi >= 0; qi = work_after<32 / QN>(S, w, qi, lane, nq))
			quad_step<TAPE, SAMP, SF>(S, q, L, stash, lane, qi, nb, overflow);
	} else {
		const int per = (nq + S.total_warps - 1) / S.total_warps;
		const int q0 = S.sched ? gw * per : gw, qstride = S.sched ? 1 : S.total_warps;
		const int qend = S.sched ? min(nq, q0 + per) : nq;
		for (int qi = q0; qi < qend; qi += qstride) quad_step<TAPE, SAMP, SF>(S, q, L, stash, lane, qi, nb, overflow);
	}
	if (nb > 0) {
		__syncwarp();
		finish_forces<TAPE, SAMP>(S, stash, nb, lane);
	}
	work_end<WL>(S, lane);
	if (__any_sync(0xffffffffu, overflow) && lane == 0) atomicOr(S.status, ST_NEIGHBOUR_OVERFLOW);
}

// MODE 2: every policy is the global method with one ORCA cost (the ORCA
// solve only: 64 registers, 8 blocks per SM, against 128 and 4 for MODE 0).
// MODE 3: every policy samples a regular schedule with one Karamouzas cost
// (the general sampler compiled out: 21% faster than MODE 0 on a 100k-agent
// corridor at the same 128 registers; at 96 registers it spilled and was
// slower).
template <int MODE, bool TAPE = false, bool OBST = true, bool SAMP = false>
__global__ void __launch_bounds__(128, MODE == 1 ? 8 : (MODE == 2 ? 8 : 4)) k_agent(DevState S, int dump)
{
	extern __shared__ unsigned char smem[];
	const int lane = threadIdx.x & 31;
	const int wib = threadIdx.x >> 5;
	const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
	const int maxnb = S.maxnb;
	uint32_t* base = reinterpret_cast<uint32_t*>(smem) + (size_t)wib * 4 * maxnb;
	WarpLists L{ base, reinterpret_cast<float*>(base + maxnb), reinterpret_cast<int*>(base + 2 * maxnb),
	             reinterpret_cast<float*>(base + 3 * maxnb) };
	bool overflow = false;
	if constexpr (MODE == 1) {
		float* stash = reinterpret_cast<float*>(smem) + (size_t)(blockDim.x >> 5) * 4 * maxnb + wib * 32 * STASH_STRIDE;
		force_agents<TAPE, OBST, SAMP>(S, L, stash, lane, gw, &overflow);
		if (overflow && lane == 0) atomicOr(S.status, ST_NEIGHBOUR_OVERFLOW);
		return;
	}
	float* fx = reinterpret_cast<float*>(L.nid);   // per-neighbour terms
	float* fy = L.aux;
	float4* lines = S.scratch + (size_t)gw * 2 * maxnb;
	float4* proj = lines + maxnb;

	WorkIter w;
	const int n_items = S.t_end - S.t_begin;
	for (int it = work_first<8>(S, w, n_items, gw, lane); it >= 0; it = work_after<8>(S, w, it, lane, n_items)) {
		const int t = S.t_begin + it;
		const int slot = S.sSlot[t];
		const float4 sb = S.sB[t];
		const float4 prm = S.prm[slot];
		const int pi = S.pol[slot];
		const PolicyDesc& pol = S.pols[pi];
		AgentCtx A;
		A.pos = S.sP[t]; A.vel = S.sV[t]; A.pref = V(sb.x, sb.y); A.goal = S.goal[slot];
		A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
		const int sc = S.agent_scen[slot];
		const ScenDesc sd = S.scen[sc];
		const GridParams G = S.grid[sc];
		A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;

		const int K = gather(S, G, S.cell_base[sc], sd.world, sd.width, sd.height, L, t, A.pos, pol.range, lane, &overflow);
		NbView N;
		N.ref = L.ref; N.d2 = L.key; N.K = K; N.sP = S.sP; N.sV = S.sV; N.sB = S.sB; N.sE = S.sE;
		N.W = sd.width; N.H = sd.height;
		N.edges = S.edges; N.obs = nullptr; N.KO = 0;

		if (dump) {
			const int cap = S.dump_cap;
			for (int k = lane; k < K && k < cap; k += 32) {
				S.dump_ids[(size_t)slot * cap + k] = S.sId[L.ref[k] & 0x0FFFFFFFu];
				S.dump_d2[(size_t)slot * cap + k] = L.key[k];
			}
			if (lane == 0) S.dump_cnt[slot] = K;
			__syncwarp();
			continue;
		}
		if (TAPE) {
			for (int k = lane; k < K; k += 32) {
				const uint32_t rr = L.ref[k];
				S.tape_list[(size_t)slot * maxnb + k] = (rr & 0xF0000000u) | (uint32_t)S.sSlot[rr & 0x0FFFFFFFu];
			}
			if (lane == 0) S.tape_cnt[slot] = K;
		}
		if (OBST && sd.nedges > 0) {
			uint32_t* ol = S.obs_list + (size_t)gw * S.max_obs;
			N.KO = gather_obstacles(S, sd, A.pos, pol.range, lane, ol);
			N.obs = ol;
		}

		// phase 5: contact forces (policy.cpp:107-141), independent of phase 4
		float2 contact = V(0, 0);
		if (pol.contact_scale > 0) {
			for (int b0 = 0; b0 < K; b0 += 32) {
				const int k = b0 + lane;
				bool take = false;
				float2 f = V(0, 0);
				if (k < K) {
					// d2[k] is |pos - neighbour|^2 computed exactly as vsq(diff); if it
					// exceeds (r + r_j)^2 by 1e-5 relative, sqrt(d2) >= r + r_j and the
					// overlap test below is false
					const float rsum = A.radius + nb_radius(N, k);
					if (!(N.d2[k] > rsum * rsum * 1.00001f)) {
						const float2 diff = vsub(A.pos, nb_pos(N, k));
						const float inter = rsum - vmag(diff);
						if (inter > 0) { take = true; f = vmul(vnorm(diff), pol.contact_scale * inter); }
					}
				}
				contact = ordered_accumulate(contact, f, take);
			}
			// colliding obstacle edges, after the agents (policy.cpp:126-137)
			for (int b0 = 0; b0 < N.KO; b0 += 32) {
				const int k = b0 + lane;
				bool take = false;
				float2 f = V(0, 0);
				if (k < N.KO) {
					float2 a, b;
					nb_seg(N, k, &a, &b);
					const float2 diff = vsub(A.pos, nearest_on_segment(A.pos, a, b));
					const float inter = A.radius - vmag(diff);
					if (inter > 0) { take = true; f = vmul(vnorm(diff), pol.contact_scale * inter); }
				}
				contact = ordered_accumulate(contact, f, take);
			}
		}

		// phase 4: Policy::ComputeNewVelocity (policy.cpp:43-76)
		float2 nv = V(0, 0);
		uint32_t rng_next = 0;
		bool rng_used = false;
		if (MODE == 2 && !viszero(A.pref)) {
			// global method, one ORCA cost: its solution (ORCA::GetGlobalMinimum)
			int nl = 0;
			const float2 best = orca_solve(A, N, pol.cost[0], lines, proj, &nl, lane);
			const float2 acc = vclamp(vdiv(vsub(best, A.vel), fmaxr(pol.relax_time, A.dt)), A.maxacc);
			nv = vclamp(vadd(A.vel, vmul(acc, A.dt)), A.maxspeed);
		} else if (MODE == 3 && !viszero(A.pref)) {
			// sampling a regular schedule with one Karamouzas cost
			CostPrep P;
			P.lines = lines; P.nlines = 0; P.orca_v = V(0, 0);
			karamouzas_prep(A, N, pol.cost[0], 0, lane, &P);
			const float2 best = sample_min<true>(S, A, N, pol, P, S.rng[slot], lane, lines, reinterpret_cast<float*>(proj));
			const float2 acc = vclamp(vdiv(vsub(best, A.vel), fmaxr(pol.relax_time, A.dt)), A.maxacc);
			nv = vclamp(vadd(A.vel, vmul(acc, A.dt)), A.maxspeed);
		} else if (MODE == 0 && !viszero(A.pref)) {
			CostPrep P;
			P.lines = lines; P.nlines = 0; P.orca_v = V(0, 0);
			for (int ci = 0; ci < pol.ncost; ++ci) {
				const CostDesc& c = pol.cost[ci];
				if (is_force_based(c.kind)) P.target[ci] = target_velocity(A, N, c, lane, fx, fy);
				else if (c.kind == K_KARAMOUZAS) karamouzas_prep(A, N, c, ci, lane, &P);
				else if (c.kind == K_ORCA) {
					P.orca_v = orca_solve(A, N, c, lines, proj, &P.nlines, lane);
				}
			}
			float2 acc;
			if (pol.method == M_GRADIENT) {
				// Policy::getAccelerationFromGradient: policy.cpp:78-89
				float2 T = V(0, 0);
				int grad_draws = 0;
				for (int ci = 0; ci < pol.ncost; ++ci) {
					const CostDesc& c = pol.cost[ci];
					float2 g;
					if (is_force_based(c.kind)) g = vdiv(vsub(A.vel, P.target[ci]), A.dt);
					else if (c.kind == K_RANDOM) {
						// RandomFunction::GetGradient (RandomFunction.cpp:30-33): two
						// numbers in [-1, 1]; the reference build evaluates the
						// constructor's second argument first
						const uint32_t r0 = S.rng[slot];
						const float gy = rng_uniform(mulmod(S.lcgpow[grad_draws + 1], r0), -1, 1);
						const float gx = rng_uniform(mulmod(S.lcgpow[grad_draws + 2], r0), -1, 1);
						grad_draws += 2;
						g = V(gx, gy);
					} else if (c.kind == K_GENERIC) g = V(0, 0);   // FD of a zero cost
					else if (c.kind == K_TTCADCA)
						g = grad_ttcadca(A, N, c, A.vel, lane, fx, fy, reinterpret_cast<float*>(proj));
					else if (c.kind == K_FOE) g = grad_foe(A, N, c, A.vel, lane, fx, fy);
					else if (c.kind >= K_PLUGIN0 &&
					         plugin_gradient(c.kind - K_PLUGIN0, A, N, c, A.vel, lane, fx, fy, &g)) {
						// the plugin's GetGradient
					} else {
						// CostFunction::GetGradient default: costFunction.cpp:36-54;
						// lanes 0..3 evaluate the four probes
						const float d = 0.1f;
						const int which = lane & 3;
						float2 probe = A.vel;
						if (which == 0) probe = vsub(A.vel, V(d, 0));
						else if (which == 1) probe = vadd(A.vel, V(d, 0));
						else if (which == 2) probe = vsub(A.vel, V(0, d));
						else probe = vadd(A.vel, V(0, d));
						const float cv = eval_cost(A, N, c, P, ci, probe);
						const float cl = __shfl_sync(0xffffffffu, cv, 0), cr = __shfl_sync(0xffffffffu, cv, 1);
						const float cb = __shfl_sync(0xffffffffu, cv, 2), ct = __shfl_sync(0xffffffffu, cv, 3);
						g = V((cr - cl) / (2 * d), (ct - cb) / (2 * d));
					}
					T = vadd(T, vmul(g, c.coeff));
				}
				acc = vmul(T, -1);
				if (TAPE && lane == 0) S.tape_acc[slot] = acc;
				if (grad_draws > 0) {
					rng_used = true;
					rng_next = mulmod(S.lcgpow[grad_draws], S.rng[slot]);
				}
			} else {
				float2 best;
				const CostDesc& c0 = pol.cost[0];
				if (pol.method == M_GLOBAL && pol.ncost == 1 && c0.kind == K_ORCA) best = P.orca_v;
				else if (pol.method == M_GLOBAL && pol.ncost == 1 && is_force_based(c0.kind)) best = P.target[0];
				else if (pol.method == M_GLOBAL && pol.ncost == 1 && c0.kind >= K_PLUGIN0 &&
				         plugin_global_minimum(c0.kind - K_PLUGIN0, A, N, c0, lane, &best)) {
					// the plugin's GetGlobalMinimum
				}
				else {
					const uint32_t r0 = S.rng[slot];
					best = sample_min(S, A, N, pol, P, r0, lane, lines, reinterpret_cast<float*>(proj));
					if (pol.draws > 0) {
						rng_used = true;
						rng_next = mulmod(S.lcgpow[pol.nsamples * pol.draws], r0);
					}
				}
				acc = vdiv(vsub(best, A.vel), fmaxr(pol.relax_time, A.dt));
			}
			acc = vclamp(acc, A.maxacc);
			nv = vclamp(vadd(A.vel, vmul(acc, A.dt)), A.maxspeed);
		}

		// phase 6: Agent::UpdateVelocityAndPosition (agent.cpp:71-93)
		if (lane == 0) {
			update_agent(S, sd, slot, A.pos, A.pref, A.dt, nv, contact);
			if (rng_used) S.rng[slot] = rng_next;
		}
		__syncwarp();
	}
	work_end(S, lane);
	if (overflow && lane == 0) atomicOr(S.status, ST_NEIGHBOUR_OVERFLOW);
}

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

// ------------------------------------------------------------------------
// differentiable form
// ------------------------------------------------------------------------
// Adjoint of one step for policies made of SocialForcesAvoidance, PowerLaw
// and GoalReachingForce under the gradient method, with the neighbour lists
// the forward step recorded.  One warp per agent (list order): the forward
// quantities are recomputed, then the adjoints of the agent's new position
// and velocity are propagated to its own state, its neighbours' states
// (atomicAdd) and the scenario's parameters (V0, sigma, k, tau0).
// Per-agent terms that the neighbours' adjoints read, from the state at the
// start of the step being reversed: the normalised goal direction Eb (as the
// scatter computes it for SocialForcesAvoidance), 1/|goal - pos| (0 at the
// goal: Eb is then constant) and the speed.
__global__ void k_adj_prep(DevState S)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= S.n) return;
	const float2 d = vsub(S.goal[i], S.a_pos[i]);
	const float4 prm = S.prm[i];
	const float2 v = S.a_vel[i];
	float2 eb = V(0, 0);
	float invw = 0;
	if (!(vsq(d) <= prm.x * prm.x)) {
		eb = vnorm(vmul(vnorm(d), prm.y));
		if (!viszero(eb)) invw = 1.0f / vmag(d);
	}
	S.adj_nb[i] = make_float4(eb.x, eb.y, invw, vmag(v));
}

// Adjoint of one step for policies made of SocialForcesAvoidance, PowerLaw
// and GoalReachingForce under the gradient method, with the neighbour lists
// the forward step recorded.  One warp per agent (list order), one lane per
// neighbour: the pair's force adjoints (every cost) and contact adjoint are
// formed together, the agent's own terms summed over the warp, and the
// neighbour's terms added to its adjoint with one atomic per nonzero
// component.  The parameters' adjoints (V0, sigma, k, tau0) are summed per
// scenario.
// this lane's share of the obstacle terms of an agent's position adjoint:
// SocialForces obstacle forces (compute_force) and contact with edges, over
// the edge list regathered from the reversed step's start state (not
// inlined, to keep k_adjoint's registers for scenarios without obstacles)
__device__ __noinline__ float2 obstacle_adjoint(const DevState& S, const ScenDesc& sd, const PolicyDesc& pol,
                                                const AgentCtx& A, int gw, int lane, bool moving, bool contact,
                                                float2 la, float2 lC)
{
	NbView N;
	N.edges = S.edges; N.W = sd.width; N.H = sd.height;
	uint32_t* ol = S.obs_list + (size_t)gw * S.max_obs;
	N.obs = ol;
	N.KO = gather_obstacles(S, sd, A.pos, pol.range, lane, ol);
	float2 lp = v2(0, 0);
	for (int k = lane; k < N.KO; k += 32) {
		float2 a, b;
		nb_seg(N, k, &a, &b);
		const EdgeSeen es = edge_seen(A.pos, a, b);
		if (moving)
			for (int c = 0; c < pol.ncost; ++c) {
				const CostDesc& cd = pol.cost[c];
				if (cd.kind != K_SOCIALFORCES || dist2_to_segment(A.pos, a, b) > cd.range * cd.range) continue;
				lp = add2(lp, sf_obstacle_adj(A, cd, es, mul2(la, cd.coeff / cd.p[5])));
			}
		if (contact) lp = add2(lp, edge_contact_adj(es, A.radius, pol.contact_scale, lC));
	}
	__syncwarp();
	return lp;
}

template <bool OBST>
__global__ void __launch_bounds__(128, 5) k_adjoint(DevState S)   // 5 blocks per SM (the launch)
{
	const int lane = threadIdx.x & 31;
	const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int nw = (gridDim.x * blockDim.x) >> 5;
	for (int i = gw; i < S.n; i += nw) {
		const int sc = S.agent_scen[i];
		const ScenDesc sd = S.scen[sc];
		const PolicyDesc& pol = S.pols[S.pol[i]];
		const float4 prm = S.prm[i];
		AgentCtx A;
		A.pos = S.a_pos[i]; A.vel = S.a_vel[i]; A.goal = S.goal[i];
		A.radius = prm.x; A.prefspeed = prm.y; A.maxspeed = prm.z; A.maxacc = prm.w;
		A.dt = sd.dt; A.relax = pol.relax_time; A.ex = S.expx;
		const float dt = sd.dt;
		const float2 lp = S.lam_out_p[i], lvo = S.lam_out_v[i];
		// p' = p + v'' dt, v'' = v' + C dt / 80
		const float2 lvn = add2(lvo, mul2(lp, dt));
		// per-lane partial adjoints, warp-summed at the end (lane 0 holds the
		// agent's own terms)
		float2 lpi = lane == 0 ? lp : v2(0, 0), lvi = v2(0, 0);
		const float2 lC = mul2(lvn, dt / 80.0f);
		// preferred velocity (agent.cpp:52-59)
		const float2 w = sub2(A.goal, A.pos);
		const bool at_goal = dot2(w, w) <= A.radius * A.radius;
		A.pref = at_goal ? v2(0, 0) : vmul(vnorm(w), A.prefspeed);
		const bool moving = !viszero(A.pref);
		const int K = S.tape_cnt[i];
		const uint32_t* list = S.tape_list + (size_t)i * S.maxnb;
		// a = sum coeff F / m (ForceBasedFunction::GetGradient with
		// policy.cpp:78-89); the forward step recorded a before the clamp
		float2 la = v2(0, 0);
		if (moving) {
			const float2 a = S.tape_acc[i];
			const float2 ac = vclamp(a, A.maxacc);
			const float2 u = add2(A.vel, mul2(ac, dt));
			const float2 lu = clamp_adj(u, A.maxspeed, lvn);
			if (lane == 0) lvi = add2(lvi, lu);
			la = clamp_adj(a, A.maxacc, mul2(lu, dt));
		}
		float2 lpref = v2(0, 0);
		float dV0 = 0, dsig = 0, dk = 0, dtau0 = 0;
		for (int c = 0; c < pol.ncost; ++c) {
			const CostDesc& cd = pol.cost[c];
			if (cd.kind == K_GOALREACHING && lane == 0) {
				const float2 lF = mul2(la, cd.coeff / cd.p[5]);
				const float mr = fmaxr(A.relax, dt);
				lpref = add2(lpref, mul2(lF, 1.0f / mr));
				lvi = sub2(lvi, mul2(lF, 1.0f / mr));
			}
		}
		const bool contact = pol.contact_scale > 0;
		if (moving || contact) {
			for (int k = lane; k < K; k += 32) {
				const uint32_t e = list[k];
				const int j = (int)(e & 0x0FFFFFFFu);
				const float2 pj = add2(S.a_pos[j], group_offset(e >> 28, sd.width, sd.height));
				const float2 D = sub2(A.pos, pj);
				const float d2 = dot2(D, D);
				const float rj = S.prm[j].x;
				float2 lpj = v2(0, 0), lvj = v2(0, 0);
				if (moving) {
					const float2 vj = S.a_vel[j];
					const float4 nb = S.adj_nb[j];
					for (int c = 0; c < pol.ncost; ++c) {
						const CostDesc& cd = pol.cost[c];
						if (cd.kind == K_GOALREACHING || d2 > cd.range * cd.range) continue;
						const float2 lF = mul2(la, cd.coeff / cd.p[5]);
						if (cd.kind == K_SOCIALFORCES) {
							const float2 ebj = v2(nb.x, nb.y);
							const SfAdj r = sf_pair_adj(A, cd, pj, vj, ebj, rj, lF);
							lpi = add2(lpi, r.lR);
							lpj = sub2(lpj, r.lR);
							lvj = add2(lvj, r.lvj);
							// Eb_j = (g_j - p_j)/|g_j - p_j| away from the goal
							lpj = sub2(lpj, mul2(sub2(r.lEb, mul2(ebj, dot2(ebj, r.lEb))), nb.z));
							dV0 += r.lV0;
							dsig += r.lsigma;
						} else {
							const PlAdj r = pl_pair_adj(A, cd, pj, vj, rj, lF);
							lpi = add2(lpi, r.lx);
							lpj = sub2(lpj, r.lx);
							lvi = add2(lvi, r.lv);
							lvj = sub2(lvj, r.lv);
							dk += r.lk;
							dtau0 += r.ltau0;
						}
					}
				}
				// contact forces (all neighbours): C = sum scale (rsum - |D|) D/|D|
				if (contact) {
					const float2 lD = contact_adj(D, A.radius + rj, pol.contact_scale, lC);
					lpi = add2(lpi, lD);
					lpj = sub2(lpj, lD);
				}
				if (lpj.x != 0) atomicAdd(&S.lam_in_p[j].x, lpj.x);
				if (lpj.y != 0) atomicAdd(&S.lam_in_p[j].y, lpj.y);
				if (lvj.x != 0) atomicAdd(&S.lam_in_v[j].x, lvj.x);
				if (lvj.y != 0) atomicAdd(&S.lam_in_v[j].y, lvj.y);
			}
		}
		// static obstacle edges (the list recomputed from the state the step
		// started from, as the forward step gathered it): SocialForces
		// obstacle forces (compute_force) and contact with edges
		if (OBST && sd.nedges > 0 && (moving || contact))
			lpi = add2(lpi, obstacle_adjoint(S, sd, pol, A, gw, lane, moving, contact, la, lC));
		// warp sums (lane 0 also holds the goal-force terms)
		float vals[8] = { lpi.x, lpi.y, lvi.x, lvi.y, dV0, dsig, dk, dtau0 };
		for (int q = 0; q < 8; ++q)
			for (int o = 16; o > 0; o >>= 1) vals[q] += __shfl_xor_sync(0xffffffffu, vals[q], o);
		if (lane == 0) {
			float2 P = v2(vals[0], vals[1]);
			if (!at_goal) P = sub2(P, mul2(normalize_adj(w, lpref), A.prefspeed));   // pref = s (g - p)/|g - p|
			atomicAdd(&S.lam_in_p[i].x, P.x); atomicAdd(&S.lam_in_p[i].y, P.y);
			atomicAdd(&S.lam_in_v[i].x, vals[2]); atomicAdd(&S.lam_in_v[i].y, vals[3]);
			float* dp = S.dparams + 4 * sc;
			if (vals[4] != 0) atomicAdd(dp + 0, vals[4]);
			if (vals[5] != 0) atomicAdd(dp + 1, vals[5]);
			if (vals[6] != 0) atomicAdd(dp + 2, vals[6]);
			if (vals[7] != 0) atomicAdd(dp + 3, vals[7]);
		}
		__syncwarp();
	}
}

// loss += w |p - target|^2 summed over agents (double accumulation)
__global__ void k_loss(DevState S, const float2* target, float w, double* loss)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	float v = 0;
	if (i < S.n) {
		const float2 d = sub2(S.pos[i], target[i]);
		v = w * dot2(d, d);
	}
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	if ((threadIdx.x & 31) == 0 && v != 0) atomicAdd(loss, (double)v);
}

// lam_p = lam_p_in + 2 w (pos - target); lam_v = lam_v_in
__global__ void k_inject(int n, const float2* pos, const float2* target, float w, const float2* lpin,
                         const float2* lvin, float2* lpout, float2* lvout)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const float2 d = sub2(pos[i], target[i]);
	lpout[i] = add2(lpin[i], mul2(d, 2 * w));
	lvout[i] = lvin[i];
}

// GetAgentPositions (APIFunctions.cpp:90-115): one record per agent
// The AgentData records (28 bytes: id, position, velocity, viewing
// direction) move through shared memory, so that the block's stretch of
// records is read or written as consecutive 4-byte words: coalesced, also
// when the buffer is page-locked host memory that the kernel accesses
// directly.
constexpr int PACK_BLOCK = 256, REC_WORDS = (int)(sizeof(AgentRecord) / 4);
static_assert(sizeof(AgentRecord) == 28, "AgentData layout");

// GetAgentPositions (APIFunctions.cpp:88-115): the records of slots [0, n)
__global__ void __launch_bounds__(PACK_BLOCK) k_pack(DevState S, AgentRecord* dst)
{
	__shared__ uint32_t w[PACK_BLOCK * REC_WORDS];
	const int i0 = blockIdx.x * PACK_BLOCK, i = i0 + threadIdx.x;
	const int cnt = min(PACK_BLOCK, S.n - i0);
	if (i < S.n) {
		const float2 p = S.pos[i], v = S.vel[i], vw = S.view[i];
		uint32_t* r = w + threadIdx.x * REC_WORDS;
		r[0] = (uint32_t)S.id[i];
		r[1] = __float_as_uint(p.x); r[2] = __float_as_uint(p.y);
		r[3] = __float_as_uint(v.x); r[4] = __float_as_uint(v.y);
		r[5] = __float_as_uint(vw.x); r[6] = __float_as_uint(vw.y);
	}
	__syncthreads();
	uint32_t* out = reinterpret_cast<uint32_t*>(dst) + (size_t)i0 * REC_WORDS;
	for (int k = threadIdx.x; k < cnt * REC_WORDS; k += PACK_BLOCK) out[k] = w[k];
}

// SetAgentPositions (APIFunctions.cpp:117-137): Agent::setPosition and
// Agent::setVelocity_ExternalApplication for every listed id that exists
__global__ void __launch_bounds__(PACK_BLOCK) k_unpack(DevState S, const AgentRecord* src, int m)
{
	__shared__ uint32_t w[PACK_BLOCK * REC_WORDS];
	const int k0 = blockIdx.x * PACK_BLOCK, k = k0 + threadIdx.x;
	const int cnt = min(PACK_BLOCK, m - k0);
	const uint32_t* in = reinterpret_cast<const uint32_t*>(src) + (size_t)k0 * REC_WORDS;
	for (int j = threadIdx.x; j < cnt * REC_WORDS; j += PACK_BLOCK) w[j] = in[j];
	__syncthreads();
	if (k >= m) return;
	const uint32_t* r = w + threadIdx.x * REC_WORDS;
	const int id = (int)r[0];
	if (id < 0 || id >= S.id_bound) return;
	const int i = S.slot_of_id[id];
	if (i < 0) return;
	S.pos[i] = V(__uint_as_float(r[1]), __uint_as_float(r[2]));
	S.vel[i] = V(__uint_as_float(r[3]), __uint_as_float(r[4]));
	S.vwf[i] = V(__uint_as_float(r[3]), __uint_as_float(r[4]));
	S.view[i] = V(__uint_as_float(r[5]), __uint_as_float(r[6]));
}

// ------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------
template <class T> static bool dalloc(T*& p, size_t n, std::string& err)
{
	if (p) cudaFree(p);
	p = nullptr;
	cudaError_t e = cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1));
	if (e != cudaSuccess) { err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return false; }
	return true;
}

Engine* Engine::create(const std::string& xml, std::string& err, const EngineOptions& opt)
{
	return create_batch(std::vector<std::string>{ xml }, err, opt);
}

Engine* Engine::create_batch(const std::vector<std::string>& xmls, std::string& err, const EngineOptions& opt)
{
	Engine* e = new Engine();
	if (!e->init(xmls, opt)) {
		err = e->err_;
		delete e;
		return nullptr;
	}
	return e;
}

static uint32_t minstd_seed(uint64_t s)
{
	uint32_t x = (uint32_t)(s % LCG_M);
	return x == 0 ? 1u : x;
}

bool Engine::init(const std::vector<std::string>& xmls, const EngineOptions& opt)
{
	opt_ = opt;
	if (xmls.empty()) { err_ = "no scenario"; return false; }
	scs_.resize(xmls.size());
	for (size_t k = 0; k < xmls.size(); ++k) {
		if (!load_scenario(xmls[k], scs_[k], err_)) {
			if (xmls.size() > 1) err_ = xmls[k] + ": " + err_;
			return false;
		}
		for (const auto& p : scs_[k].policies) {
			int norca = 0;
			for (int c = 0; c < p.ncost; ++c) norca += p.cost[c].kind == K_ORCA;
			if (norca > 1) { err_ = "a policy with more than one ORCA cost function is not supported"; return false; }
		}
	}
	sc_ = scs_[0];
	int dev = 0;
	CK(cudaGetDevice(&dev));
	CK(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
	CK(cudaFuncSetAttribute(k_scan_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scan_smem_bytes(SCAN_SMEM_MAX_CELLS)));
	CK(cudaFuncSetAttribute(k_count_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scan_smem_bytes(SCAN_SMEM_MAX_CELLS)));
	CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
	CK(cudaMallocHost(&status_host_, sizeof(int)));
	for (cudaEvent_t* e : { &ev0_, &ev1_, &pa0_, &pa1_, &ps0_, &ps1_ }) CK(cudaEventCreate(e));
	d_ = new DevState();
	std::memset(d_, 0, sizeof(DevState));
	d_->cells_per_range = opt_.cells_per_range;
	d_->nscen = (int)scs_.size();
	next_unused_id_ = sc_.next_unused_id;
	// agents present at time 0, scenario by scenario, each in the order the
	// reference adds them; policies concatenated with a base per scenario
	scen_.resize(scs_.size());
	for (size_t k = 0; k < scs_.size(); ++k) {
		const Scenario& sc = scs_[k];
		const int pbase = (int)pols_.size();
		for (const auto& p : sc.policies) { pols_.push_back(p); pol_scen_.push_back((int)k); }
		ScenDesc& D = scen_[k];
		D.world = sc.world; D.width = sc.width; D.height = sc.height; D.dt = sc.dt;
		D.edge_off = (int)edges_.size();
		D.nedges = (int)sc.edges.size();
		edges_.insert(edges_.end(), sc.edges.begin(), sc.edges.end());
		float mr = 0;
		for (const auto& p : sc.policies) mr = std::max(mr, p.range);
		D.max_range = mr;
		D.agent_off = (int)id_.size();
		for (const auto& a : sc.agents) {
			if (a.start_time > 0) {
				AgentInit p = a;
				p.scen = (int)k;
				p.policy += pbase;
				pending_.push_back(p);
				continue;
			}
			if (k == 0) slot_of_[a.id] = (int)id_.size();
			id_.push_back(a.id); pol_.push_back(pbase + a.policy);
			agent_scen_.push_back((int)k);
			pos_.push_back(make_float2(a.x, a.y)); vel_.push_back(make_float2(0, 0));
			goal_.push_back(make_float2(a.gx, a.gy)); vwf_.push_back(make_float2(0, 0));
			prm_.push_back(make_float4(a.radius, a.pref_speed, a.max_speed, a.max_accel));
			rng_.push_back(minstd_seed((unsigned int)a.id));
			remove_.push_back(a.remove_at_goal ? 1 : 0);
			// Agent::setGoal: agent.cpp:108-115
			float2 v0 = make_float2(0, 0);
			if (a.gx != a.x || a.gy != a.y) {
				float dx = a.gx - a.x, dy = a.gy - a.y, m = sqrtf(dx * dx + dy * dy);
				if (m > 0) { dx = dx / m; dy = dy / m; }
				v0 = make_float2(dx, dy);
			}
			view_.push_back(v0);
			any_remove_at_goal_ |= a.remove_at_goal;
		}
		D.n = (int)id_.size() - D.agent_off;
		D.max_cells = scs_.size() == 1 ? std::max(4096, std::min(1 << 24, 4 * D.n + 1024)) : 4 * D.n + 256;
	}
	std::stable_sort(pending_.begin(), pending_.end(),
	                 [](const AgentInit& x, const AgentInit& y) { return x.start_time < y.start_time; });
	for (const auto& a : pending_) any_remove_at_goal_ |= a.remove_at_goal;
	n_ = (int)id_.size();
	times_.assign(scs_.size(), 0.0);
	bool need_exp = false;
	for (const auto& p : pols_)
		for (int c = 0; c < p.ncost; ++c)
			need_exp |= p.cost[c].kind == K_SOCIALFORCES || p.cost[c].kind == K_POWERLAW || p.cost[c].kind == K_FOE ||
			            p.cost[c].kind >= K_PLUGIN0;   // a plugin may call ref_expf
	if (need_exp && !exp_exceptions_for_device(&d_->expx, nullptr, err_)) return false;
	// kernel groups: scenarios whose policies have force-based costs only
	// (k_force_quad or k_agent<1>, whatever the method), scenarios with an
	// ORCA cost, the others (k_agent<0>); cell space orders scenarios by group
	{
		std::vector<int> cls(scen_.size(), 0);
		std::vector<char> pure_orca(scen_.size(), 1);   // every policy: global method, one ORCA cost
		std::vector<char> pure_kara(scen_.size(), 1);   // every policy: regular sampling, one Karamouzas cost
		for (size_t k = 0; k < scen_.size(); ++k) {
			bool force_only = true, orca = false;
			for (size_t pi = 0; pi < pols_.size(); ++pi) {
				if (pol_scen_[pi] != (int)k) continue;
				const PolicyDesc& P = pols_[pi];
				if (!(P.method == M_GLOBAL && P.ncost == 1 && P.cost[0].kind == K_ORCA)) pure_orca[k] = 0;
				if (!(P.method == M_SAMPLING && P.ncost == 1 && P.cost[0].kind == K_KARAMOUZAS && P.s_type == 0))
					pure_kara[k] = 0;
				// any method: the force-only kernels pick the velocity from the
				// cost targets (gradient step, global minimum or sample argmin)
				for (int c = 0; c < P.ncost; ++c) {
					const int kd = P.cost[c].kind;
					if (!(kd == K_SOCIALFORCES || kd == K_POWERLAW || kd == K_GOALREACHING)) force_only = false;
					if (kd == K_ORCA) orca = true;
				}
			}
			cls[k] = force_only ? 0 : (orca ? 1 : 2);
		}
		scen_order_.clear();
		groups_.clear();
		for (int c = 0; c < 3; ++c) {
			const int j0 = (int)scen_order_.size();
			for (size_t k = 0; k < scen_.size(); ++k)
				if (cls[k] == c) scen_order_.push_back((int)k);
			if ((int)scen_order_.size() > j0) {
				KGroup g{ c == 0 ? 1 : 0, j0, (int)scen_order_.size(), 0, 0, 0 };
				if (c == 1) {
					bool all = true;
					for (int j = j0; j < g.j1; ++j) all = all && pure_orca[scen_order_[j]];
					if (all) g.mode = 2;   // k_agent<2>: the ORCA-only kernel
				} else if (c == 2) {
					bool all = true;
					for (int j = j0; j < g.j1; ++j) all = all && pure_kara[scen_order_[j]];
					if (all) g.mode = 3;   // k_agent<3>: the Karamouzas-sampling kernel
				}
				for (int j = j0; j < g.j1; ++j) g.obst |= scen_[scen_order_[j]].nedges > 0;
				g.quad_ok = g.mode == 1 && !g.obst;
				g.samp = false;
				g.sf_only = true;
				for (size_t pi = 0; pi < pols_.size(); ++pi) {
					bool in_group = false;
					for (int j = j0; j < g.j1; ++j) in_group |= pol_scen_[pi] == scen_order_[j];
					if (!in_group) continue;
					int nbc = 0;
					for (int c2 = 0; c2 < pols_[pi].ncost; ++c2) nbc += pols_[pi].cost[c2].kind != K_GOALREACHING;
					if (nbc > 1) g.quad_ok = false;
					for (int c2 = 0; c2 < pols_[pi].ncost; ++c2) {
						const int kd = pols_[pi].cost[c2].kind;
						if (kd != K_GOALREACHING && kd != K_SOCIALFORCES) g.sf_only = false;
					}
					if (pols_[pi].method != M_GRADIENT) g.samp = true;
				}
				groups_.push_back(g);
			}
		}
		if (!dalloc(scen_order_dev_, scen_order_.size(), err_)) return false;
		CK(cudaMemcpy(scen_order_dev_, scen_order_.data(), sizeof(int) * scen_order_.size(), cudaMemcpyHostToDevice));
		d_->scen_order = scen_order_dev_;
		toric_only_ = !scen_.empty();
		for (const auto& D : scen_) toric_only_ = toric_only_ && D.world == W_TORIC;
		static_grid_ready_ = false;
	}
	if (!edges_.empty()) {
		if (!dalloc(edges_dev_, edges_.size(), err_)) return false;
		CK(cudaMemcpy(edges_dev_, edges_.data(), sizeof(float4) * edges_.size(), cudaMemcpyHostToDevice));
	}
	d_->edges = edges_dev_;
	build_edge_grids();
	if (!og_items_.empty()) {
		if (!dalloc(og_start_dev_, og_start_.size(), err_) || !dalloc(og_items_dev_, og_items_.size(), err_) ||
		    !dalloc(og_ecell_dev_, og_ecell_.size(), err_))
			return false;
		CK(cudaMemcpy(og_start_dev_, og_start_.data(), sizeof(int) * og_start_.size(), cudaMemcpyHostToDevice));
		CK(cudaMemcpy(og_items_dev_, og_items_.data(), sizeof(int2) * og_items_.size(), cudaMemcpyHostToDevice));
		CK(cudaMemcpy(og_ecell_dev_, og_ecell_.data(), sizeof(int4) * og_ecell_.size(), cudaMemcpyHostToDevice));
	}
	d_->og_start = og_start_dev_;
	d_->og_items = og_items_dev_;
	d_->og_ecell = og_ecell_dev_;
	if (!build_tables()) return false;
	// the host sinf/cosf: random-sample rotations (build_tables), the gradient
	// rotations of TtcaDca and FOEAvoidance, the segment collision times
	bool need_trig = need_trig_ || !edges_.empty();
	for (const auto& p : pols_)
		for (int c = 0; c < p.ncost; ++c)
			need_trig |= p.cost[c].kind == K_TTCADCA || p.cost[c].kind == K_FOE ||
			             p.cost[c].kind >= K_PLUGIN0;   // a plugin may call host_sinf / host_sincosf
	if (need_trig && !set_device_sincos(err_)) return false;
	if (!alloc(std::max(n_, 16))) return false;
	if (!upload_all()) return false;
	if (!choose_maxnb()) return false;
	return true;
}

// Edge grids of the scenarios with many obstacle edges (host, once): cell size
// the scenario's largest interaction range (doubled until the grid has at
// most 4 cells per edge + 1024), each edge listed in every cell its bounding
// box overlaps, in edge order.
void Engine::build_edge_grids()
{
	og_start_.clear();
	og_items_.clear();
	og_ecell_.assign(edges_.size(), make_int4(0, 0, -1, -1));
	for (auto& D : scen_) {
		D.og_nx = D.og_ny = 0;
		if (D.nedges < OBS_GRID_MIN_EDGES) continue;
		float x0 = FLT_MAX, y0 = FLT_MAX, x1 = -FLT_MAX, y1 = -FLT_MAX;
		for (int k = 0; k < D.nedges; ++k) {
			const float4 e = edges_[D.edge_off + k];
			x0 = std::min(x0, std::min(e.x, e.z)); x1 = std::max(x1, std::max(e.x, e.z));
			y0 = std::min(y0, std::min(e.y, e.w)); y1 = std::max(y1, std::max(e.y, e.w));
		}
		if (!(x1 >= x0 && y1 >= y0) || !std::isfinite(x1 - x0) || !std::isfinite(y1 - y0)) continue;
		float cs = std::max(D.max_range, 1e-3f);
		while (((double)(x1 - x0) / cs + 1.0) * ((double)(y1 - y0) / cs + 1.0) > 4.0 * D.nedges + 1024) cs *= 2.0f;
		const float inv = 1.0f / cs;
		const int nx = (int)((x1 - x0) * inv) + 1, ny = (int)((y1 - y0) * inv) + 1;
		std::vector<std::vector<int2>> cells((size_t)nx * ny);
		for (int k = 0; k < D.nedges; ++k) {
			const float4 e = edges_[D.edge_off + k];
			const int4 c = make_int4(obs_cell(std::min(e.x, e.z), x0, inv, nx), obs_cell(std::min(e.y, e.w), y0, inv, ny),
			                         obs_cell(std::max(e.x, e.z), x0, inv, nx), obs_cell(std::max(e.y, e.w), y0, inv, ny));
			og_ecell_[D.edge_off + k] = c;
			for (int cy = c.y; cy <= c.w; ++cy)
				for (int cx = c.x; cx <= c.z; ++cx) cells[(size_t)cy * nx + cx].push_back(make_int2(D.edge_off + k, cx));
		}
		D.og_x0 = x0; D.og_y0 = y0; D.og_inv = inv; D.og_nx = nx; D.og_ny = ny;
		// og_start_[D.og_start + cell] .. [+ 1]: the cell's items (absolute)
		D.og_start = (int)og_start_.size();
		for (const auto& c : cells) {
			og_start_.push_back((int)og_items_.size());
			og_items_.insert(og_items_.end(), c.begin(), c.end());
		}
		og_start_.push_back((int)og_items_.size());
	}
}

bool Engine::build_tables()
{
	std::vector<PolicyDesc> pols = pols_;
	std::vector<SampleEntry> table;
	size_t maxdraws = 0;   // random numbers an agent draws in one step, over all policies
	for (auto& p : pols) {
		p.use_sampling = 0; p.table_random = 0; p.single_cost = 0;
		p.table_offset = 0; p.nsamples = 0; p.len_divisor = 1;
		p.nrand = 0; p.draws = 0;
		for (int c = 0; c < p.ncost; ++c) p.nrand += p.cost[c].kind == K_RANDOM;
		// RandomFunction::GetGradient draws two numbers per cost (RandomFunction.cpp:30-33)
		if (p.method == M_GRADIENT) maxdraws = std::max(maxdraws, (size_t)(2 * p.nrand));
		bool sampling = p.method == M_SAMPLING;
		int type = p.s_type, base = p.s_base, dir = p.s_dir, rad = p.s_radius, ns = p.speed_samples, na = p.angle_samples,
		    incl = p.include_base;
		float angle = p.s_angle;
		if (p.method == M_GLOBAL) {
			const int k0 = p.cost[0].kind;
			const bool closed = p.ncost == 1 && (k0 == K_ORCA || k0 == K_SOCIALFORCES || k0 == K_POWERLAW || k0 == K_GOALREACHING);
			if (!closed) {
				// SamplingParameters::ApproximateGlobalOptimization: policy.h:74-86
				sampling = true;
				type = 0; base = 0; dir = 0; rad = 1; angle = 360; na = 36; ns = 11; incl = 1;
				p.single_cost = p.ncost == 1 ? 1 : 0;
			}
		}
		if (!sampling) continue;
		if (p.single_cost) p.nrand = p.cost[0].kind == K_RANDOM ? 1 : 0;
		p.use_sampling = 1;
		p.table_base = base; p.table_dir = dir; p.table_radius = rad;
		p.max_angle = (float)(angle / 360.0 * 3.1415926535897);
		if (type == 1) {
			// random sampling (costFunction.cpp:99-119): angle, then length, then
			// one number per RandomFunction cost, sample after sample
			p.table_random = 1;
			p.nsamples = std::max(p.random_samples, 0);
			p.draws = 2 + p.nrand;
			maxdraws = std::max(maxdraws, (size_t)p.nsamples * p.draws);
			continue;
		}
		// regular schedule: costFunction.cpp:122-158 (float angle accumulation)
		p.table_offset = (int)table.size();
		const float maxAngle = p.max_angle;
		const float startAngle = -maxAngle, endAngle = maxAngle;
		const float deltaAngle = (endAngle - startAngle) / (float)(angle == 360 ? na : (na - 1));
		p.len_divisor = incl ? (ns - 1) : ns;
		for (int s = 1; s <= ns; ++s) {
			float a = startAngle;
			for (int k = 0; k < na; ++k, a += deltaAngle) {
				SampleEntry e;
				e.c = cosf(a); e.s = sinf(a);
				e.mult = (float)(incl ? s - 1 : s);
				e.pad = 0;
				table.push_back(e);
				if (incl && s == 1) break;
			}
		}
		p.nsamples = (int)table.size() - p.table_offset;
		p.draws = p.nrand;
		maxdraws = std::max(maxdraws, (size_t)p.nsamples * p.draws);
	}
	if (table.empty()) table.push_back(SampleEntry{ 0, 0, 0, 0 });
	need_trig_ = false;
	for (const auto& p : pols) need_trig_ |= p.table_random != 0;
	std::vector<uint32_t> pw(maxdraws + 3);
	pw[0] = 1;
	for (size_t k = 1; k < pw.size(); ++k) pw[k] = (uint32_t)(((uint64_t)pw[k - 1] * LCG_A) % LCG_M);
	PolicyDesc* dp = nullptr;
	SampleEntry* dt = nullptr;
	uint32_t* dl = nullptr;
	if (!dalloc(dp, pols.size(), err_) || !dalloc(dt, table.size(), err_) || !dalloc(dl, pw.size(), err_)) return false;
	CK(cudaMemcpy(dp, pols.data(), sizeof(PolicyDesc) * pols.size(), cudaMemcpyHostToDevice));
	CK(cudaMemcpy(dt, table.data(), sizeof(SampleEntry) * table.size(), cudaMemcpyHostToDevice));
	CK(cudaMemcpy(dl, pw.data(), sizeof(uint32_t) * pw.size(), cudaMemcpyHostToDevice));
	d_->pols = dp; d_->table = dt; d_->lcgpow = dl;
	return true;
}

bool Engine::alloc(int cap)
{
	cap_ = cap;
	DevState& S = *d_;
	if (scen_.size() == 1) scen_[0].max_cells = std::max(4096, std::min(1 << 24, 4 * cap + 1024));
	int64_t mc = 0;
	for (const auto& D : scen_) mc += D.max_cells;
	if (mc > (1 << 28)) { err_ = "too many grid cells"; return false; }
	S.max_cells = (int)mc;
	const int ns = (int)scen_.size();
	if (!dalloc(S.pos, cap, err_) || !dalloc(S.vel, cap, err_) || !dalloc(S.goal, cap, err_) ||
	    !dalloc(S.view, cap, err_) || !dalloc(S.vwf, cap, err_) || !dalloc(S.pref, cap, err_) ||
	    !dalloc(S.prm, cap, err_) || !dalloc(S.pol, cap, err_) || !dalloc(S.id, cap, err_) ||
	    !dalloc(S.rng, cap, err_) || !dalloc(S.sP, cap, err_) || !dalloc(S.sV, cap, err_) ||
	    !dalloc(S.sB, cap, err_) || !dalloc(S.sE, cap, err_) || !dalloc(S.sSlot, cap, err_) || !dalloc(S.sId, cap, err_) ||
	    !dalloc(S.cell, cap, err_) || !dalloc(S.agent_scen, cap, err_) || !dalloc(S.cnt, mc + 1, err_) ||
	    !dalloc(S.start, mc + 1, err_) ||
	    !dalloc(S.blocksum, mc / SCAN_PER_BLOCK + 5, err_))
		return false;
	S.ticket = reinterpret_cast<unsigned*>(S.blocksum + mc / SCAN_PER_BLOCK + 2);
	S.gbar = reinterpret_cast<unsigned*>(S.blocksum + mc / SCAN_PER_BLOCK + 3);
	CK(cudaMemset(S.ticket, 0, 3 * sizeof(unsigned)));
	if (!S.grid && !dalloc(S.grid, ns, err_)) return false;
	if (!S.bbox && !dalloc(S.bbox, 4 * ns, err_)) return false;
	if (!S.cell_base && !dalloc(S.cell_base, ns + 1, err_)) return false;
	if (!S.status) {
		if (!dalloc(S.status, 1, err_)) return false;
		CK(cudaMemset(S.status, 0, sizeof(int)));
	}
	CK(cudaMemset(S.cnt, 0, sizeof(int) * (mc + 1)));
	// bbox sentinels: min = +FLT_MAX, max = -FLT_MAX in ordered encoding
	auto enc = [](float f) { unsigned u; std::memcpy(&u, &f, 4); return (u & 0x80000000u) ? ~u : (u | 0x80000000u); };
	std::vector<unsigned> hb(4 * ns);
	for (int k = 0; k < ns; ++k) { hb[4 * k] = hb[4 * k + 1] = enc(FLT_MAX); hb[4 * k + 2] = hb[4 * k + 3] = enc(-FLT_MAX); }
	CK(cudaMemcpy(S.bbox, hb.data(), sizeof(unsigned) * hb.size(), cudaMemcpyHostToDevice));
	invalidate_graph();
	return true;
}

bool Engine::upload_all()
{
	DevState& S = *d_;
	S.n = n_;
	if (n_ > 0) {
		CK(cudaMemcpy(S.pos, pos_.data(), sizeof(float2) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.vel, vel_.data(), sizeof(float2) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.goal, goal_.data(), sizeof(float2) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.view, view_.data(), sizeof(float2) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.vwf, vwf_.data(), sizeof(float2) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.prm, prm_.data(), sizeof(float4) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.pol, pol_.data(), sizeof(int) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.id, id_.data(), sizeof(int) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.rng, rng_.data(), sizeof(uint32_t) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.agent_scen, agent_scen_.data(), sizeof(int) * n_, cudaMemcpyHostToDevice));
	}
	// scenario 0 owns every agent of a single simulation (including agents
	// added or removed later)
	if (scen_.size() == 1) { scen_[0].agent_off = 0; scen_[0].n = n_; }
	if (!scen_dev_ && !dalloc(scen_dev_, scen_.size(), err_)) return false;
	CK(cudaMemcpy(scen_dev_, scen_.data(), sizeof(ScenDesc) * scen_.size(), cudaMemcpyHostToDevice));
	S.scen = scen_dev_;
	int bound = 1;
	for (int v : id_) bound = std::max(bound, v + 1);
	std::vector<int> so(bound, -1);
	for (int i = 0; i < n_; ++i) so[id_[i]] = i;
	if (bound > S.id_bound || !S.slot_of_id) {
		if (!dalloc(S.slot_of_id, (size_t)std::max(bound, 2 * S.id_bound), err_)) return false;
	}
	S.id_bound = bound;
	CK(cudaMemcpy(S.slot_of_id, so.data(), sizeof(int) * bound, cudaMemcpyHostToDevice));
	if (!dalloc(S.io, (size_t)std::max(cap_, 1), err_)) return false;
	invalidate_graph();
	return true;
}

// true when p is page-locked (or registered) host memory
static bool is_pinned(const void* p)
{
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeHost;
}

// The device's address of page-locked host memory (kernels read and write it
// directly), or null for other memory
static void* host_device_view(const void* p)
{
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Page-locked staging for AgentData exchange with pageable caller buffers:
// a host copy into it plus a page-locked transfer beats the driver's
// pageable path.
bool Engine::stage(size_t records)
{
	if (records <= io_host_cap_) return true;
	if (io_host_) cudaFreeHost(io_host_);
	io_host_ = nullptr;
	io_host_cap_ = 0;
	CK(cudaMallocHost(&io_host_, sizeof(AgentRecord) * records));
	io_host_cap_ = records;
	return true;
}

bool Engine::get_agent_data(void* out)
{
	DevState& S = *d_;
	if (!sync()) return false;
	if (n_ == 0) return true;
	S.n = n_;
	const int nb = (n_ + PACK_BLOCK - 1) / PACK_BLOCK;
	const size_t bytes = sizeof(AgentRecord) * n_;
	// page-locked output: the kernel writes it directly
	if (AgentRecord* dv = static_cast<AgentRecord*>(host_device_view(out))) {
		k_pack<<<nb, PACK_BLOCK, 0, stream_>>>(S, dv);
		CK(cudaGetLastError());
		CK(cudaStreamSynchronize(stream_));
		return true;
	}
	if (!stage(n_)) return false;
	AgentRecord* sv = static_cast<AgentRecord*>(host_device_view(io_host_));
	if (sv) {
		k_pack<<<nb, PACK_BLOCK, 0, stream_>>>(S, sv);
	} else {
		k_pack<<<nb, PACK_BLOCK, 0, stream_>>>(S, S.io);
		CK(cudaMemcpyAsync(io_host_, S.io, bytes, cudaMemcpyDeviceToHost, stream_));
	}
	CK(cudaGetLastError());
	CK(cudaStreamSynchronize(stream_));
	std::memcpy(out, io_host_, bytes);
	return true;
}

bool Engine::set_agent_data(const void* in, int m)
{
	DevState& S = *d_;
	if (!sync()) return false;
	if (m <= 0) return true;
	const size_t bytes = sizeof(AgentRecord) * m;
	const int nb = (m + PACK_BLOCK - 1) / PACK_BLOCK;
	// page-locked input: the kernel reads it directly
	if (const AgentRecord* dv = static_cast<const AgentRecord*>(host_device_view(in))) {
		k_unpack<<<nb, PACK_BLOCK, 0, stream_>>>(S, dv, m);
		CK(cudaGetLastError());
		CK(cudaStreamSynchronize(stream_));
		return true;
	}
	if (!stage(m)) return false;
	std::memcpy(io_host_, in, bytes);
	const AgentRecord* sv = static_cast<const AgentRecord*>(host_device_view(io_host_));
	if (sv) {
		k_unpack<<<nb, PACK_BLOCK, 0, stream_>>>(S, sv, m);
	} else {
		if (m > cap_ && !dalloc(S.io, (size_t)m, err_)) return false;
		CK(cudaMemcpyAsync(S.io, io_host_, bytes, cudaMemcpyHostToDevice, stream_));
		k_unpack<<<nb, PACK_BLOCK, 0, stream_>>>(S, S.io, m);
	}
	CK(cudaGetLastError());
	CK(cudaStreamSynchronize(stream_));
	if (!sv && m > cap_ && !dalloc(S.io, (size_t)std::max(cap_, 1), err_)) return false;
	return true;
}

bool Engine::download_mutable()
{
	const DevState& S = *d_;
	if (!sync()) return false;
	pos_.resize(n_); vel_.resize(n_); view_.resize(n_); vwf_.resize(n_); rng_.resize(n_);
	if (n_ > 0) {
		CK(cudaMemcpy(pos_.data(), S.pos, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(vel_.data(), S.vel, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(view_.data(), S.view, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(vwf_.data(), S.vwf, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(rng_.data(), S.rng, sizeof(uint32_t) * n_, cudaMemcpyDeviceToHost));
	}
	return true;
}

// The neighbour-list capacity is sized from the initial state: one and a
// half times the largest list plus 16, rounded up to a multiple of 32 (at
// least 64), which keeps the lists of four agents per warp within shared
// memory at full occupancy.  A list that later outgrows it sets
// ST_NEIGHBOUR_OVERFLOW; sync() then re-runs the batch from its snapshot with
// the capacity grown by half (up to 3072 entries): shared memory per block,
// and so occupancy, follows the capacity.
static int grown_capacity(int c)
{
	return std::min(3072, std::max(c + 32, (c + c / 2 + 31) / 32 * 32));
}

bool Engine::choose_maxnb()
{
	int want = opt_.max_neighbours;
	if (want <= 0) {
		const int probe = 3072;
		std::vector<int> cnt(std::max(n_, 1));
		int saved = maxnb_;
		maxnb_ = probe;
		if (!neighbours(0, nullptr, nullptr, cnt.data())) { maxnb_ = saved; return false; }
		int mx = 0;
		for (int i = 0; i < n_; ++i) mx = std::max(mx, cnt[i]);
		want = std::max(64, std::min(3072, (mx + mx / 2 + 16 + 31) / 32 * 32));
	}
	if (want != maxnb_) {
		maxnb_ = want;
		invalidate_graph();
	}
	return true;
}

void Engine::invalidate_graph()
{
	if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
	if (graph_) cudaGraphDestroy(graph_);
	graph_exec_ = nullptr;
	graph_ = nullptr;
	graph_valid_ = false;
}

// Dynamic shared memory of a k_agent launch: per warp the four neighbour
// lists, and for the force-only kernel its per-lane agent records.
static size_t agent_smem(int warps_per_block, int maxnb, int mode)
{
	size_t b = (size_t)warps_per_block * maxnb * 16;
	if (mode == 1) b += (size_t)warps_per_block * 32 * STASH_STRIDE * sizeof(float);
	return b;
}

// k_force_quad: per warp four agents' lists (reference, key) and the agent records
static size_t quad_smem(int warps_per_block, int maxnb)
{
	return (size_t)warps_per_block * (QN * q_words(maxnb) + 32 * STASH_STRIDE) * sizeof(float);
}

static int quad_blocks_for(int num_sms, int warps_per_block, size_t smem)
{
	int per_sm = 0;
	cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_force_quad<false>, warps_per_block * 32, smem);
	if (per_sm < 1) per_sm = 1;
	return num_sms * per_sm;
}

static int agent_blocks_for(int num_sms, int warps_per_block, size_t smem, int mode = 0, bool obst = true)
{
	int per_sm = 0;
	if (mode == 2)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agent<2>, warps_per_block * 32, smem);
	else if (mode == 3)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agent<3>, warps_per_block * 32, smem);
	else if (mode == 1 && !obst)
		cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agent<1, false, false>, warps_per_block * 32, smem);
	else if (mode == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agent<1>, warps_per_block * 32, smem);
	else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_agent<0>, warps_per_block * 32, smem);
	if (per_sm < 1) per_sm = 1;
	return num_sms * per_sm;
}

// Launch shape of k_agent for the current neighbour capacity: as many
// 4-warp blocks as fit on every SM, and ORCA line scratch for each warp.
bool Engine::configure()
{
	DevState& S = *d_;
	const int wpb = opt_.warps_per_block;
	const size_t smem0 = agent_smem(wpb, maxnb_, 0), smem1 = agent_smem(wpb, maxnb_, 1);
	const size_t smemq = quad_smem(wpb, maxnb_);
	if (smemq > 48 * 1024) {
		CK(cudaFuncSetAttribute(k_force_quad<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
		CK(cudaFuncSetAttribute(k_force_quad<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
		CK(cudaFuncSetAttribute(k_force_quad<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
		CK(cudaFuncSetAttribute(k_force_quad<true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
		CK(cudaFuncSetAttribute(k_force_quad<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
		CK(cudaFuncSetAttribute(k_force_quad<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
		CK(cudaFuncSetAttribute(k_force_quad<false, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
		CK(cudaFuncSetAttribute(k_force_quad<false, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemq));
	}
	if (smem0 > 48 * 1024) {
		CK(cudaFuncSetAttribute(k_agent<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0));
		CK(cudaFuncSetAttribute(k_agent<0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0));
		CK(cudaFuncSetAttribute(k_agent<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0));
		CK(cudaFuncSetAttribute(k_agent<2, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0));
		CK(cudaFuncSetAttribute(k_agent<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0));
		CK(cudaFuncSetAttribute(k_agent<3, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0));
	}
	if (smem1 > 48 * 1024) {
		CK(cudaFuncSetAttribute(k_agent<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
		CK(cudaFuncSetAttribute(k_agent<1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
		CK(cudaFuncSetAttribute(k_agent<1, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
		CK(cudaFuncSetAttribute(k_agent<1, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
		CK(cudaFuncSetAttribute(k_agent<1, false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
		CK(cudaFuncSetAttribute(k_agent<1, false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
	}
	mode_ = 1;
	for (const auto& g : groups_) if (g.mode != 1) mode_ = 0;
	// one launch shape per kernel group, each with its own line scratch
	size_t scr = 0, obs = 0;
	int maxe = 0;
	for (const auto& D : scen_) maxe = std::max(maxe, D.nedges);
	S.max_obs = 5 * maxe;   // every edge, once per displacement group
	for (auto& g : groups_) {
		g.quad = g.quad_ok && opt_.agent_lanes == 8;
		g.blocks = g.quad ? quad_blocks_for(num_sms_, wpb, smemq)
		                  : agent_blocks_for(num_sms_, wpb, g.mode == 1 ? smem1 : smem0, g.mode, g.obst);
		if (opt_.occupancy < 1.0f) g.blocks = std::max(num_sms_, (int)(g.blocks * opt_.occupancy));
		g.scratch_off = scr;
		scr += (size_t)g.blocks * wpb * 2 * maxnb_;
		g.obs_off = obs;
		obs += (size_t)g.blocks * wpb * S.max_obs;
	}
	if (!dalloc(S.obs_list, std::max<size_t>(obs, 1), err_)) return false;
	agent_blocks_ = groups_.empty() ? num_sms_ : groups_[0].blocks;
	S.total_warps = agent_blocks_ * wpb;
	S.sched = opt_.schedule;
	S.cells_per_range = opt_.cells_per_range;
	static_grid_ready_ = false;   // the cell size may have changed
	if (!dalloc(S.scratch, std::max<size_t>(scr, 1), err_)) return false;
	// work-list counters: a pair per kernel group, and one for the list dump
	if (!dalloc(S.work, 2 * (groups_.size() + 1), err_)) return false;
	CK(cudaMemset(S.work, 0, sizeof(unsigned) * 2 * (groups_.size() + 1)));
	configured_maxnb_ = maxnb_;
	invalidate_graph();
	return true;
}

void Engine::enqueue_step()
{
	DevState& S = *d_;
	S.n = n_;
	S.maxnb = maxnb_;
	const int wpb = opt_.warps_per_block;
	const size_t smem0 = agent_smem(wpb, maxnb_, 0), smem1 = agent_smem(wpb, maxnb_, 1);
	const size_t smemq = quad_smem(wpb, maxnb_);
	S.counters = profile_ ? counters_ : nullptr;
	enqueue_grid(S);
	if (profile_) cudaEventRecord(pa0_, stream_);
	// the agents of each kernel group form one range of the cell-sorted
	// arrays (scenarios are ordered by group in cell space)
	int t = 0;
	std::vector<int> tb(groups_.size()), te(groups_.size());
	for (size_t k = 0; k < groups_.size(); ++k) {
		const KGroup& g = groups_[k];
		int cnt = 0;
		if (scen_.size() == 1) cnt = n_;
		else for (int j = g.j0; j < g.j1; ++j) cnt += scen_[scen_order_[j]].n;
		tb[k] = t; te[k] = t + cnt; t += cnt;
	}
	auto launch = [&](size_t k, cudaStream_t st) {
		const KGroup& g = groups_[k];
		if (te[k] <= tb[k]) return;
		DevState A = S;
		A.t_begin = tb[k]; A.t_end = te[k];
		// no more blocks than the group has agents for (small worlds)
		const int per_block = g.quad ? wpb * QN : wpb;
		const int blocks = std::min(g.blocks, std::max(1, (te[k] - tb[k] + per_block - 1) / per_block));
		A.total_warps = blocks * wpb;
		A.work = S.work + 2 * k;
		A.scratch = S.scratch + g.scratch_off;
		A.obs_list = S.obs_list + g.obs_off;
		if (g.quad) {
			// taped runs are gradient-only (diff_begin checks)
			const bool wl = S.sched == 2;
			if (S.tape_list) {
				if (wl) k_force_quad<true, false, true><<<blocks, wpb * 32, smemq, st>>>(A);
				else k_force_quad<true><<<blocks, wpb * 32, smemq, st>>>(A);
			} else if (g.samp) {
				if (wl) k_force_quad<false, true, true><<<blocks, wpb * 32, smemq, st>>>(A);
				else k_force_quad<false, true><<<blocks, wpb * 32, smemq, st>>>(A);
			} else if (g.sf_only) {
				if (wl) k_force_quad<false, false, true, true><<<blocks, wpb * 32, smemq, st>>>(A);
				else k_force_quad<false, false, false, true><<<blocks, wpb * 32, smemq, st>>>(A);
			} else if (wl) k_force_quad<false, false, true><<<blocks, wpb * 32, smemq, st>>>(A);
			else k_force_quad<false><<<blocks, wpb * 32, smemq, st>>>(A);
		} else if (g.mode == 2) {   // taped runs have no ORCA policy (diff_begin checks)
			if (g.obst) k_agent<2><<<blocks, wpb * 32, smem0, st>>>(A, 0);
			else k_agent<2, false, false><<<blocks, wpb * 32, smem0, st>>>(A, 0);
		} else if (g.mode == 3) {   // nor a sampling one
			if (g.obst) k_agent<3><<<blocks, wpb * 32, smem0, st>>>(A, 0);
			else k_agent<3, false, false><<<blocks, wpb * 32, smem0, st>>>(A, 0);
		} else if (g.mode == 1 && g.samp && !S.tape_list) {
			if (g.obst) k_agent<1, false, true, true><<<blocks, wpb * 32, smem1, st>>>(A, 0);
			else k_agent<1, false, false, true><<<blocks, wpb * 32, smem1, st>>>(A, 0);
		} else if (S.tape_list) {
			if (g.mode == 1 && g.obst) k_agent<1, true, true><<<blocks, wpb * 32, smem1, st>>>(A, 0);
			else if (g.mode == 1) k_agent<1, true, false><<<blocks, wpb * 32, smem1, st>>>(A, 0);
			else k_agent<0, true><<<blocks, wpb * 32, smem0, st>>>(A, 0);
		} else if (g.mode == 1 && g.obst) k_agent<1, false, true><<<blocks, wpb * 32, smem1, st>>>(A, 0);
		else if (g.mode == 1) k_agent<1, false, false><<<blocks, wpb * 32, smem1, st>>>(A, 0);
		else k_agent<0><<<blocks, wpb * 32, smem0, st>>>(A, 0);
	};
	// one after the other: each launch fills the GPU (measured: running the
	// groups on concurrent streams was no faster)
	for (size_t k = 0; k < groups_.size(); ++k) launch(k, stream_);
	if (profile_) cudaEventRecord(pa1_, stream_);
}

bool Engine::small_world() const
{
	return scen_.size() == 1 && n_ <= SMALL_MAX_AGENTS && d_->max_cells <= SMALL_MAX_CELLS;
}

// The grid build: one block for a small single-scenario world; else the
// bounding box and grid parameters (every step in infinite worlds; once, by
// ensure_static_grid, when every world is toric: its grid is the world
// box), the histogram, the scan (one block up to SCAN_SINGLE_MAX_CELLS
// cells) and the scatter.
void Engine::enqueue_grid(const DevState& S)
{
	if (small_world()) {
		k_build_small<<<1, 1024, 0, stream_>>>(S);
		return;
	}
	const int threads = 256;
	const int nb = std::max(1, (n_ + threads - 1) / threads);
	const bool grid_fixed = toric_only_ && static_grid_ready_;
	if (!grid_fixed) {
		k_bbox<<<nb, threads, 0, stream_>>>(S);
		k_grid<<<1, 1024, 0, stream_>>>(S);
	}
	const int cells_bound = grid_fixed ? static_cells_ : S.max_cells;
	if (grid_fixed && coop_state_ > 0) {
		launch_grid_coop(S);   // a launch error is caught after the step is enqueued
		return;
	}
	if (grid_fixed && cells_bound <= SCAN_SMEM_MAX_CELLS) {
		k_count_scan<<<std::max(1, (n_ + 1023) / 1024), 1024, scan_smem_bytes(cells_bound), stream_>>>(S, cells_bound);
		k_scatter<<<nb, threads, 0, stream_>>>(S);
		return;
	}
	k_count<<<nb, threads, 0, stream_>>>(S);
	if (cells_bound <= SCAN_SMEM_MAX_CELLS) {
		k_scan_smem<<<1, 1024, scan_smem_bytes(cells_bound), stream_>>>(S, cells_bound);
	} else if (cells_bound <= SCAN_SINGLE_MAX_CELLS) {
		k_scan_single<<<1, 1024, 0, stream_>>>(S);
	} else {
		const int sb = (S.max_cells + SCAN_PER_BLOCK - 1) / SCAN_PER_BLOCK;
		k_scan_reduce<<<sb, SCAN_BLOCK, 0, stream_>>>(S);
		k_scan_top<<<1, 1024, 0, stream_>>>(S);
		k_scan_down<<<sb, SCAN_BLOCK, 0, stream_>>>(S);
	}
	k_scatter<<<nb, threads, 0, stream_>>>(S);
}

// The one-launch grid build (k_grid_coop): one block per SM (the agents
// spread over all of them, one per thread), blocks of up to 1024 threads,
// more blocks only when the agents need them (at most as many as are
// resident at once).
cudaError_t Engine::launch_grid_coop(const DevState& S)
{
	const int threads = std::min(1024, std::max(32, (n_ + num_sms_ - 1) / num_sms_ + 31) / 32 * 32);
	const int want = std::max(1, (n_ + threads - 1) / threads);
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)std::min(want, coop_blocks_max_));
	cfg.blockDim = dim3(threads);
	cfg.dynamicSmemBytes = 0;
	cfg.stream = stream_;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeCooperative;
	attr[0].val.cooperative = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, k_grid_coop, S);
}

// Once, outside any capture: whether the cooperative launch can be captured
// into a graph (a throwaway capture, never launched).  If not, the static
// grid is built in two launches.
void Engine::probe_grid_coop()
{
	if (coop_state_ != 0) return;
	coop_state_ = -1;
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_grid_coop, 1024, 0) != cudaSuccess || per_sm < 1) {
		cudaGetLastError();
		return;
	}
	coop_blocks_max_ = per_sm * num_sms_;
	if (cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
		cudaGetLastError();
		return;
	}
	const cudaError_t e = launch_grid_coop(*d_);
	cudaGraph_t g = nullptr;
	const cudaError_t e2 = cudaStreamEndCapture(stream_, &g);
	if (g) cudaGraphDestroy(g);
	cudaGetLastError();
	if (e == cudaSuccess && e2 == cudaSuccess) coop_state_ = 1;
}

// Toric worlds only: the grid parameters and cell ranges, which do not
// change between steps, computed once outside any graph capture.
bool Engine::ensure_static_grid()
{
	if (!toric_only_ || static_grid_ready_ || small_world()) return true;
	probe_grid_coop();
	DevState& S = *d_;
	S.n = n_;
	k_grid<<<1, 1024, 0, stream_>>>(S);
	CK(cudaGetLastError());
	CK(cudaMemcpyAsync(&static_cells_, S.cell_base + scen_.size(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
	CK(cudaStreamSynchronize(stream_));
	static_grid_ready_ = true;
	invalidate_graph();
	return true;
}

void Engine::set_profile(bool on)
{
	profile_ = on;
	prof_agent_ms_ = prof_step_ms_ = prof_grid_ms_ = 0;
	prof_steps_ = 0;
	if (on) {
		if (!counters_ && cudaMalloc(&counters_, 3 * sizeof(unsigned long long)) != cudaSuccess) counters_ = nullptr;
		if (counters_) cudaMemsetAsync(counters_, 0, 3 * sizeof(unsigned long long), stream_);
	}
}

bool Engine::profile_counters(unsigned long long* out, int n)
{
	for (int k = 0; k < n; ++k) out[k] = 0;
	if (!counters_) return true;
	unsigned long long c[3];
	CK(cudaMemcpy(c, counters_, sizeof(c), cudaMemcpyDeviceToHost));
	for (int k = 0; k < n && k < 3; ++k) out[k] = c[k];
	return true;
}

int Engine::kernels_per_step() const
{
	if (small_world()) return 1 + (int)groups_.size();
	const bool grid_fixed = toric_only_ && static_grid_ready_;
	const int cells_bound = grid_fixed ? static_cells_ : d_->max_cells;
	if (grid_fixed && coop_state_ > 0) return 1 + (int)groups_.size();
	if (grid_fixed && cells_bound <= SCAN_SMEM_MAX_CELLS) return 2 + (int)groups_.size();
	const bool single = cells_bound <= SCAN_SINGLE_MAX_CELLS;
	return (grid_fixed ? 0 : 2) + 1 + (single ? 1 : 3) + 1 + (int)groups_.size();
}

bool Engine::capture_graph()
{
	invalidate_graph();
	CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
	enqueue_step();
	cudaError_t e = cudaStreamEndCapture(stream_, &graph_);
	if (e != cudaSuccess) { err_ = std::string("graph capture: ") + cudaGetErrorString(e); return false; }
	CK(cudaGraphInstantiate(&graph_exec_, graph_, 0));
	graph_valid_ = true;
	return true;
}

// Host copy of the per-agent arrays in list order, rebuilt scenario by
// scenario when agents join or leave (order within a scenario as the
// reference's agent list).
struct Engine::AgentLists {
	std::vector<int> id, pol, scen;
	std::vector<unsigned char> remove;
	std::vector<float2> pos, vel, goal, view, vwf;
	std::vector<float4> prm;
	std::vector<uint32_t> rng;
};

void Engine::take_lists(AgentLists& L)
{
	L.id.swap(id_); L.pol.swap(pol_); L.scen.swap(agent_scen_); L.remove.swap(remove_);
	L.pos.swap(pos_); L.vel.swap(vel_); L.goal.swap(goal_); L.view.swap(view_); L.vwf.swap(vwf_);
	L.prm.swap(prm_); L.rng.swap(rng_);
	for (auto* v : { &id_, &pol_, &agent_scen_ }) v->clear();
	remove_.clear();
	for (auto* v : { &pos_, &vel_, &goal_, &view_, &vwf_ }) v->clear();
	prm_.clear();
	rng_.clear();
}

void Engine::append_agent(const AgentLists& L, int i)
{
	id_.push_back(L.id[i]); pol_.push_back(L.pol[i]); agent_scen_.push_back(L.scen[i]); remove_.push_back(L.remove[i]);
	pos_.push_back(L.pos[i]); vel_.push_back(L.vel[i]); goal_.push_back(L.goal[i]); view_.push_back(L.view[i]);
	vwf_.push_back(L.vwf[i]); prm_.push_back(L.prm[i]); rng_.push_back(L.rng[i]);
}

void Engine::append_new_agent(const AgentInit& a)
{
	id_.push_back(a.id); pol_.push_back(a.policy);
	agent_scen_.push_back(a.scen);
	pos_.push_back(make_float2(a.x, a.y)); vel_.push_back(make_float2(0, 0));
	goal_.push_back(make_float2(a.gx, a.gy)); vwf_.push_back(make_float2(0, 0));
	prm_.push_back(make_float4(a.radius, a.pref_speed, a.max_speed, a.max_accel));
	rng_.push_back(minstd_seed((unsigned int)a.id));
	remove_.push_back(a.remove_at_goal ? 1 : 0);
	// Agent::setGoal: agent.cpp:108-115
	float2 v0 = make_float2(0, 0);
	if (a.gx != a.x || a.gy != a.y) {
		float dx = a.gx - a.x, dy = a.gy - a.y, m = sqrtf(dx * dx + dy * dy);
		if (m > 0) { dx = dx / m; dy = dy / m; }
		v0 = make_float2(dx, dy);
	}
	view_.push_back(v0);
}

// The clock of scenario k (a single simulation's own time)
double Engine::scen_time(int k) const { return scen_.size() == 1 ? time_ : times_[k]; }

bool Engine::agents_due() const
{
	for (const auto& a : pending_)
		if ((double)a.start_time <= scen_time(a.scen)) return true;
	return false;
}

// After a change of the agent list: scenario 0's id -> slot map (the single
// simulation's id lookups), the count, the capacity, the device copy.
bool Engine::finish_list_change()
{
	n_ = (int)id_.size();
	slot_of_.clear();
	const int n0 = scen_.size() == 1 ? n_ : scen_[0].n;
	for (int i = 0; i < n0; ++i) slot_of_[id_[i]] = i;
	bool grow = n_ > cap_;
	if (scen_.size() > 1) {
		// a batch scenario's cell capacity follows its population
		int64_t mc = 0;
		for (auto& D : scen_) {
			D.max_cells = std::max(D.max_cells, 4 * D.n + 256);
			mc += D.max_cells;
		}
		grow |= mc > d_->max_cells;
	}
	if (grow && !alloc(n_ > cap_ ? std::max(n_, 2 * cap_) : cap_)) return false;
	return upload_all();
}

bool Engine::apply_pending_agents()
{
	// WorldBase::DoStep: agents whose start time has come (worldBase.cpp:82-86)
	// join the end of their scenario's agent list, in start order
	if (!agents_due()) return true;
	if (!download_mutable()) return false;
	AgentLists L;
	take_lists(L);
	std::vector<AgentInit> later;
	std::vector<std::vector<AgentInit>> due(scen_.size());
	for (const auto& a : pending_) {
		if ((double)a.start_time <= scen_time(a.scen)) due[a.scen].push_back(a);
		else later.push_back(a);
	}
	for (size_t k = 0; k < scen_.size(); ++k) {
		ScenDesc& D = scen_[k];
		const int off = scen_.size() == 1 ? 0 : D.agent_off, n = scen_.size() == 1 ? (int)L.id.size() : D.n;
		D.agent_off = (int)id_.size();
		for (int i = off; i < off + n; ++i) append_agent(L, i);
		for (const auto& a : due[k]) append_new_agent(a);
		D.n = (int)id_.size() - D.agent_off;
	}
	pending_.swap(later);
	return finish_list_change();
}

bool Engine::remove_at_goal()
{
	// WorldBase::DoStep tail (worldBase.cpp:122-127): each scenario's agents
	// from the last to the first; an agent at its goal that is removed there
	// takes the place of its scenario's last agent (removeAgentAtListIndex
	// :207-235)
	if (!download_mutable()) return false;
	std::vector<std::vector<int>> keep(scen_.size());
	bool changed = false;
	for (size_t k = 0; k < scen_.size(); ++k) {
		const int off = scen_.size() == 1 ? 0 : scen_[k].agent_off, n = scen_.size() == 1 ? n_ : scen_[k].n;
		std::vector<int>& idx = keep[k];
		idx.resize(n);
		for (int i = 0; i < n; ++i) idx[i] = off + i;
		for (int i = n - 1; i >= 0; --i) {
			const int a = idx[i];
			if (!remove_[a]) continue;
			const float dx = goal_[a].x - pos_[a].x, dy = goal_[a].y - pos_[a].y;
			const float r = prm_[a].x;
			if (dx * dx + dy * dy <= r * r) {
				if (!changed && !rec_flush_async()) return false;   // the ring's agents are the old list
				idx[i] = idx.back();
				idx.pop_back();
				changed = true;
			}
		}
	}
	if (!changed) return true;
	AgentLists L;
	take_lists(L);
	for (size_t k = 0; k < scen_.size(); ++k) {
		scen_[k].agent_off = (int)id_.size();
		for (int i : keep[k]) append_agent(L, i);
		scen_[k].n = (int)id_.size() - scen_[k].agent_off;
	}
	return finish_list_change();
}

// Enqueues n steps (no host work in between).
bool Engine::run_steps(int nsteps, bool record)
{
	if (configured_maxnb_ != maxnb_ && !configure()) return false;
	if (!ensure_static_grid()) return false;
	steps_pending_ = true;
	record = record && !recs_.empty();
	if (record && n_ > rec_cap_n_) {
		// the population grew since the ring was sized (it was flushed then)
		CK(cudaStreamSynchronize(stream_));
		rec_cap_n_ = n_;
		if (!dalloc(rec_ring_, (size_t)rec_R_ * rec_cap_n_, err_)) return false;
	}
	for (int s = 0; s < nsteps; ++s) {
		if (opt_.use_graph && !profile_) {
			if (!graph_valid_ && !capture_graph()) return false;
			CK(cudaGraphLaunch(graph_exec_, stream_));
		} else {
			if (profile_) CK(cudaEventRecord(ps0_, stream_));
			enqueue_step();
			CK(cudaGetLastError());
			if (profile_) {
				CK(cudaEventRecord(ps1_, stream_));
				CK(cudaEventSynchronize(ps1_));
				float a = 0, b = 0, g = 0;
				cudaEventElapsedTime(&a, pa0_, pa1_);
				cudaEventElapsedTime(&b, ps0_, ps1_);
				cudaEventElapsedTime(&g, ps0_, pa0_);
				prof_agent_ms_ += a;
				prof_step_ms_ += b;
				prof_grid_ms_ += g;
				prof_steps_ += 1;
			}
		}
		time_ += sc_.dt;
		for (size_t k = 0; k < times_.size(); ++k) times_[k] += scen_[k].dt;
		if (record && n_ > 0) {
			// RunSimulationSteps hands the writer every agent's position after
			// each step with the world's time (crowdSimulator.cpp:81-93)
			if (rec_head_ == 0) {
				rec_ids_ = id_;
				rec_off_.resize(scen_.size() + 1);
				for (size_t k = 0; k < scen_.size(); ++k) rec_off_[k] = scen_.size() == 1 ? 0 : scen_[k].agent_off;
				rec_off_[scen_.size()] = n_;
			}
			CK(cudaMemcpyAsync(rec_ring_ + (size_t)rec_head_ * n_, d_->pos, sizeof(float2) * n_,
			                   cudaMemcpyDeviceToDevice, stream_));
			for (size_t k = 0; k < scen_.size(); ++k) rec_times_[k].push_back(scen_time((int)k));
			++rec_head_;
		}
	}
	return true;
}

// ------------------------------------------------------------------------
// trajectory output
// ------------------------------------------------------------------------
bool Engine::record_start(const std::string& dir, int ring_steps, int format)
{
	if (!sync()) return false;
	if (!recs_.empty() && !record_stop()) return false;
	if (ring_steps < 1) { err_ = "ring_steps must be positive"; return false; }
	if (scen_.size() == 1) {
		recs_.push_back(new TrajWriter(dir, format));
	} else {
		// a batch: scenario k into dir/scenario_k
		TrajWriter parent(dir, format);
		std::string e = parent.error();
		if (!e.empty()) { err_ = e; return false; }
		std::string base = dir;
		if (base.empty() || base.back() != '/') base += '/';
		for (size_t k = 0; k < scen_.size(); ++k) recs_.push_back(new TrajWriter(base + "scenario_" + std::to_string(k), format));
	}
	for (TrajWriter* w : recs_) {
		const std::string e = w->error();
		if (!e.empty()) { err_ = e; rec_free(); return false; }
	}
	rec_R_ = ring_steps;
	rec_cap_n_ = std::max(n_, 1);
	if (!dalloc(rec_ring_, (size_t)rec_R_ * rec_cap_n_, err_)) { rec_free(); return false; }
	for (int b = 0; b < 2; ++b) {
		rec_busy_[b].store(0);
		if (!rec_ev_[b]) CK(cudaEventCreateWithFlags(&rec_ev_[b], cudaEventDisableTiming));
	}
	rec_head_ = rec_snap_head_ = 0;
	rec_times_.assign(scen_.size(), {});
	return true;
}

bool Engine::rec_flush_async()
{
	if (recs_.empty() || rec_head_ == 0) return true;
	const int b = rec_next_;
	if (rec_busy_[b].load())
		for (TrajWriter* w : recs_) w->drain();
	const size_t floats = (size_t)rec_head_ * n_ * 2;
	if (rec_host_cap_[b] < floats) {
		if (rec_host_[b]) cudaFreeHost(rec_host_[b]);
		rec_host_[b] = nullptr;
		rec_host_cap_[b] = 0;
		CK(cudaMallocHost(&rec_host_[b], sizeof(float) * floats));
		rec_host_cap_[b] = floats;
	}
	CK(cudaMemcpyAsync(rec_host_[b], rec_ring_, sizeof(float) * floats, cudaMemcpyDeviceToHost, stream_));
	CK(cudaEventRecord(rec_ev_[b], stream_));
	// the ring's agents and times, scenario by scenario (the offsets of the
	// ring's first step: the list does not change while the ring fills)
	rec_busy_[b].store((int)recs_.size());
	for (size_t k = 0; k < recs_.size(); ++k) {
		const int o = rec_off_[k], m = rec_off_[k + 1] - o;
		recs_[k]->push(m, rec_head_, std::vector<int>(rec_ids_.begin() + o, rec_ids_.begin() + o + m), rec_times_[k],
		               rec_host_[b], rec_ev_[b], &rec_busy_[b], (int)rec_ids_.size(), o);
	}
	rec_head_ = rec_snap_head_ = 0;
	rec_times_.assign(scen_.size(), {});
	rec_next_ ^= 1;
	// a grown population needs a larger ring before the next step is recorded
	if (n_ > rec_cap_n_) {
		CK(cudaStreamSynchronize(stream_));
		rec_cap_n_ = n_;
		if (!dalloc(rec_ring_, (size_t)rec_R_ * rec_cap_n_, err_)) return false;
	}
	return true;
}

bool Engine::rec_before_change()
{
	if (recs_.empty() || rec_head_ == 0) return true;
	if (!sync()) return false;
	return rec_flush_async();
}

bool Engine::record_flush()
{
	if (recs_.empty()) return true;
	if (!sync()) return false;
	if (!rec_flush_async()) return false;
	for (TrajWriter* w : recs_) {
		w->drain();
		const std::string e = w->error();
		if (!e.empty()) { err_ = e; return false; }
	}
	return true;
}

bool Engine::record_stop()
{
	if (recs_.empty()) return true;
	const bool ok = record_flush();
	rec_free();
	return ok;
}

void Engine::rec_free()
{
	for (TrajWriter* w : recs_) delete w;   // drains and joins the writers
	recs_.clear();
	if (rec_ring_) cudaFree(rec_ring_);
	rec_ring_ = nullptr;
	for (int b = 0; b < 2; ++b) {
		if (rec_host_[b]) cudaFreeHost(rec_host_[b]);
		rec_host_[b] = nullptr;
		rec_host_cap_[b] = 0;
	}
	rec_head_ = rec_snap_head_ = 0;
	rec_times_.clear();
}

// The mutable per-agent state at the start of a batch of steps, kept so that
// a batch in which some neighbour list outgrew the capacity can be re-run
// with a larger capacity (every step is then computed with complete lists).
// the mutable state copied in one launch (position, velocity, view,
// velocity without forces, random state)
__global__ void k_copy_state(int n, const float2* p, const float2* v, const float2* w, const float2* f,
                             const uint32_t* r, float2* P, float2* Vv, float2* W, float2* F, uint32_t* R)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	P[i] = p[i]; Vv[i] = v[i]; W[i] = w[i]; F[i] = f[i]; R[i] = r[i];
}

bool Engine::take_snapshot()
{
	DevState& S = *d_;
	if (snap_cap_ < n_) {
		snap_cap_ = std::max(n_, 16);
		if (!dalloc(snap_pos_, snap_cap_, err_) || !dalloc(snap_vel_, snap_cap_, err_) ||
		    !dalloc(snap_view_, snap_cap_, err_) || !dalloc(snap_vwf_, snap_cap_, err_) ||
		    !dalloc(snap_rng_, snap_cap_, err_))
			return false;
	}
	if (n_ > 0) {
		k_copy_state<<<(n_ + 255) / 256, 256, 0, stream_>>>(n_, S.pos, S.vel, S.view, S.vwf, S.rng, snap_pos_, snap_vel_,
		                                                    snap_view_, snap_vwf_, snap_rng_);
		CK(cudaGetLastError());
	}
	snap_valid_ = true;
	rec_snap_head_ = rec_head_;
	snap_time_ = time_;
	snap_times_ = times_;
	snap_steps_ = 0;
	return true;
}

bool Engine::restore_snapshot()
{
	DevState& S = *d_;
	if (n_ > 0) {
		CK(cudaMemcpyAsync(S.pos, snap_pos_, sizeof(float2) * n_, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.vel, snap_vel_, sizeof(float2) * n_, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.view, snap_view_, sizeof(float2) * n_, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.vwf, snap_vwf_, sizeof(float2) * n_, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.rng, snap_rng_, sizeof(uint32_t) * n_, cudaMemcpyDeviceToDevice, stream_));
	}
	time_ = snap_time_;
	times_ = snap_times_;
	rec_head_ = rec_snap_head_;
	for (auto& t : rec_times_) t.resize(rec_head_);
	return true;
}

bool Engine::step(int nsteps)
{
	if (nsteps <= 0) return true;
	const bool dynamic = !pending_.empty() || any_remove_at_goal_;   // agents join or leave between steps
	if (time_kernels) CK(cudaEventRecord(ev0_, stream_));
	if (!dynamic) {
		// with trajectory output, batches stop where the ring is full; the
		// ring is handed over once its steps are committed
		int left = nsteps;
		while (left > 0) {
			int k = left;
			if (!recs_.empty()) {
				if (rec_head_ == rec_R_ && (!sync() || !rec_flush_async())) return false;
				k = std::min(left, rec_R_ - rec_head_);
			}
			if (!snap_valid_ && !take_snapshot()) return false;
			if (!run_steps(k, true)) return false;
			snap_steps_ += k;
			left -= k;
		}
	} else {
		// insertions and removals change the agent list between steps: settle
		// every step before the host-side changes
		for (int s = 0; s < nsteps; ++s) {
			if (!recs_.empty() && rec_head_ == rec_R_ && (!sync() || !rec_flush_async())) return false;
			if (agents_due() && !rec_before_change()) return false;
			if (!pending_.empty() && !apply_pending_agents()) return false;
			if (!take_snapshot()) return false;
			if (!run_steps(1, true)) return false;
			snap_steps_ = 1;
			if (!sync()) return false;
			if (any_remove_at_goal_ && !remove_at_goal()) return false;
		}
	}
	if (time_kernels) {
		CK(cudaEventRecord(ev1_, stream_));
		CK(cudaEventSynchronize(ev1_));
		float ms = 0;
		cudaEventElapsedTime(&ms, ev0_, ev1_);
		agent_ms_ = ms / nsteps;
	}
	return true;
}

// Waits for the enqueued steps.  A neighbour-capacity overflow restores the
// snapshot taken at the start of the batch, doubles the capacity and re-runs
// the batch; other device conditions are reported.
bool Engine::sync()
{
	if (!steps_pending_) return true;   // nothing enqueued since the last check
	for (;;) {
		// the status word follows the steps on the stream into page-locked
		// host memory: one synchronisation
		CK(cudaMemcpyAsync(status_host_, d_->status, sizeof(int), cudaMemcpyDeviceToHost, stream_));
		CK(cudaStreamSynchronize(stream_));
		const int st = *status_host_;
		if (st == 0) {
			snap_valid_ = false;
			steps_pending_ = false;
			return true;
		}
		CK(cudaMemset(d_->status, 0, sizeof(int)));
		if ((st & ST_NEIGHBOUR_OVERFLOW) && snap_valid_ && maxnb_ < 3072) {
			const int steps = snap_steps_;
			if (!restore_snapshot()) return false;
			maxnb_ = grown_capacity(maxnb_);
			invalidate_graph();
			if (!run_steps(steps, true)) return false;
			continue;
		}
		snap_valid_ = false;
		if (st & ST_NEIGHBOUR_OVERFLOW) {
			err_ = "a neighbour list is longer than " + std::to_string(maxnb_) + " entries";
			return false;
		}
		if (st & ST_GRID_OVERFLOW) { err_ = "non-finite agent positions"; return false; }
		if (st & ST_GRID_BARRIER) { err_ = "grid build: a block gave up waiting at a grid barrier"; return false; }
		err_ = "device status " + std::to_string(st);
		return false;
	}
}

bool Engine::get_state(int* ids, float* pos, float* vel, float* view, float* pref, float* goal)
{
	const DevState& S = *d_;
	if (!sync()) return false;
	if (n_ == 0) return true;
	if (ids) std::memcpy(ids, id_.data(), sizeof(int) * n_);
	if (pos) CK(cudaMemcpy(pos, S.pos, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
	if (vel) CK(cudaMemcpy(vel, S.vel, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
	if (view) CK(cudaMemcpy(view, S.view, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
	if (pref) CK(cudaMemcpy(pref, S.pref, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
	if (goal) CK(cudaMemcpy(goal, S.goal, sizeof(float2) * n_, cudaMemcpyDeviceToHost));
	return true;
}

bool Engine::set_state(const float* pos, const float* vel, const float* view)
{
	const DevState& S = *d_;
	if (!sync()) return false;
	if (n_ == 0) return true;
	if (pos) CK(cudaMemcpy(S.pos, pos, sizeof(float2) * n_, cudaMemcpyHostToDevice));
	if (vel) {
		CK(cudaMemcpy(S.vel, vel, sizeof(float2) * n_, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(S.vwf, vel, sizeof(float2) * n_, cudaMemcpyHostToDevice));
	}
	if (view) CK(cudaMemcpy(S.view, view, sizeof(float2) * n_, cudaMemcpyHostToDevice));
	return true;
}

bool Engine::set_agent_by_id(int id, float px, float py, float vx, float vy, float wx, float wy)
{
	auto it = slot_of_.find(id);
	if (it == slot_of_.end()) return true;   // SetAgentPositions skips unknown ids
	const int i = it->second;
	const DevState& S = *d_;
	float2 p = make_float2(px, py), v = make_float2(vx, vy), w = make_float2(wx, wy);
	CK(cudaMemcpyAsync(S.pos + i, &p, sizeof(float2), cudaMemcpyHostToDevice, stream_));
	CK(cudaMemcpyAsync(S.vel + i, &v, sizeof(float2), cudaMemcpyHostToDevice, stream_));
	CK(cudaMemcpyAsync(S.vwf + i, &v, sizeof(float2), cudaMemcpyHostToDevice, stream_));
	CK(cudaMemcpyAsync(S.view + i, &w, sizeof(float2), cudaMemcpyHostToDevice, stream_));
	CK(cudaStreamSynchronize(stream_));
	return true;
}

bool Engine::set_goal(int id, float x, float y)
{
	// Agent::setGoal: agent.cpp:108-115
	auto it = slot_of_.find(id);
	if (it == slot_of_.end()) { err_ = "no agent with id " + std::to_string(id); return false; }
	const int i = it->second;
	const DevState& S = *d_;
	float2 p;
	if (!sync()) return false;
	CK(cudaMemcpy(&p, S.pos + i, sizeof(float2), cudaMemcpyDeviceToHost));
	float2 g = make_float2(x, y);
	goal_[i] = g;
	CK(cudaMemcpy(S.goal + i, &g, sizeof(float2), cudaMemcpyHostToDevice));
	if (g.x != p.x || g.y != p.y) {
		float dx = g.x - p.x, dy = g.y - p.y, m = sqrtf(dx * dx + dy * dy);
		if (m > 0) { dx = dx / m; dy = dy / m; }
		float2 w = make_float2(dx, dy);
		CK(cudaMemcpy(S.view + i, &w, sizeof(float2), cudaMemcpyHostToDevice));
	}
	return true;
}

bool Engine::add_agent(float x, float y, float radius, float pref, float maxs, float maxacc, int policy_id,
                       int desired_id, int* out_id)
{
	// AddAgent (APIFunctions.cpp:139-171) -> WorldBase::AddAgent (worldBase.cpp:161-186)
	if (scen_.size() > 1) { err_ = "agents cannot be added to a batch"; return false; }
	if (!rec_before_change()) return false;
	int pidx = -1;
	for (size_t k = 0; k < sc_.policy_ids.size(); ++k)
		if (sc_.policy_ids[k] == policy_id) pidx = (int)k;
	if (pidx < 0) { err_ = "no policy with id " + std::to_string(policy_id); return false; }
	if (!download_mutable()) return false;
	int id = (desired_id >= 0 && !slot_of_.count(desired_id)) ? desired_id : next_unused_id_;
	if (id >= next_unused_id_) next_unused_id_ = id + 1;
	slot_of_[id] = (int)id_.size();
	id_.push_back(id); pol_.push_back(pidx);
	agent_scen_.push_back(0);
	pos_.push_back(make_float2(x, y)); vel_.push_back(make_float2(0, 0));
	goal_.push_back(make_float2(x, y)); vwf_.push_back(make_float2(0, 0));
	view_.push_back(make_float2(0, 0));
	prm_.push_back(make_float4(radius, pref, maxs, maxacc));
	rng_.push_back(minstd_seed((unsigned int)id));
	remove_.push_back(0);
	n_ = (int)id_.size();
	if (n_ > cap_ && !alloc(std::max(n_, 2 * cap_))) return false;
	if (!upload_all()) return false;
	if (out_id) *out_id = id;
	return true;
}

bool Engine::remove_agent(int id)
{
	// WorldBase::RemoveAgent (worldBase.cpp:198-235): the last agent moves into the gap
	if (scen_.size() > 1) { err_ = "agents cannot be removed from a batch"; return false; }
	if (!rec_before_change()) return false;
	auto it = slot_of_.find(id);
	if (it == slot_of_.end()) { err_ = "no agent with id " + std::to_string(id); return false; }
	if (!download_mutable()) return false;
	const int i = it->second, last = n_ - 1;
	slot_of_.erase(id);
	if (i != last) {
		id_[i] = id_[last]; pol_[i] = pol_[last]; pos_[i] = pos_[last]; vel_[i] = vel_[last];
		goal_[i] = goal_[last]; view_[i] = view_[last]; vwf_[i] = vwf_[last]; prm_[i] = prm_[last];
		rng_[i] = rng_[last]; remove_[i] = remove_[last];
		slot_of_[id_[i]] = i;
	}
	id_.pop_back(); pol_.pop_back(); pos_.pop_back(); vel_.pop_back(); goal_.pop_back();
	view_.pop_back(); vwf_.pop_back(); prm_.pop_back(); rng_.pop_back(); remove_.pop_back();
	agent_scen_.pop_back();
	n_ = last;
	return upload_all();
}

bool Engine::neighbours(int cap, int* ids, float* d2, int* counts)
{
	DevState& S = *d_;
	if (!sync()) return false;
	if (n_ == 0) return true;
	const int dcap = std::max(cap, 1);
	if (!dalloc(S.dump_ids, (size_t)n_ * dcap, err_) || !dalloc(S.dump_d2, (size_t)n_ * dcap, err_) ||
	    !dalloc(S.dump_cnt, n_, err_))
		return false;
	S.dump_cap = dcap;
	// same grid build and gather as a step, no state update
	DevState T = S;
	T.n = n_;
	const int dump_nb = std::max(maxnb_, 3072);   // 4 warps x 3072 x 16 B = 192 KB shared
	T.maxnb = dump_nb;
	const int wpb = opt_.warps_per_block;
	const size_t smem = (size_t)wpb * dump_nb * 16;
	if (smem > 48 * 1024) CK(cudaFuncSetAttribute(k_agent<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const int blocks = agent_blocks_for(num_sms_, wpb, smem);
	T.total_warps = blocks * wpb;
	T.work = S.work + 2 * groups_.size();
	float4* scr = nullptr;
	if (!dalloc(scr, (size_t)T.total_warps * 2 * dump_nb, err_)) return false;
	T.scratch = scr;
	if (!ensure_static_grid()) { cudaFree(scr); return false; }
	enqueue_grid(T);
	T.t_begin = 0;
	T.t_end = n_;
	k_agent<0><<<blocks, wpb * 32, smem, stream_>>>(T, 1);
	CK(cudaGetLastError());
	CK(cudaStreamSynchronize(stream_));
	cudaFree(scr);
	int st = 0;
	CK(cudaMemcpy(&st, S.status, sizeof(int), cudaMemcpyDeviceToHost));
	CK(cudaMemset(S.status, 0, sizeof(int)));
	if (counts) CK(cudaMemcpy(counts, S.dump_cnt, sizeof(int) * n_, cudaMemcpyDeviceToHost));
	if (ids && cap > 0) CK(cudaMemcpy(ids, S.dump_ids, sizeof(int) * (size_t)n_ * cap, cudaMemcpyDeviceToHost));
	if (d2 && cap > 0) CK(cudaMemcpy(d2, S.dump_d2, sizeof(float) * (size_t)n_ * cap, cudaMemcpyDeviceToHost));
	if (st & ST_NEIGHBOUR_OVERFLOW) { err_ = "neighbour list longer than " + std::to_string(dump_nb); return false; }
	// the dump kernel leaves the step's scratch sizes as they were
	return true;
}

// Chooses the launch shape of the step by timing a few steps of each
// candidate from the current state, which is restored afterwards.  Every
// candidate computes bit-identical results: the cell size changes which
// cells are scanned, not which neighbours are found or their order.
bool Engine::set_launch(const EngineOptions& o)
{
	if (!(o.cells_per_range > 0) || o.warps_per_block < 1 || o.warps_per_block > 8 || !(o.occupancy > 0) ||
	    o.occupancy > 1 || o.schedule < 0 || o.schedule > 2 || (o.agent_lanes != 8 && o.agent_lanes != 32)) {
		err_ = "launch shape out of range";
		return false;
	}
	if (!sync()) return false;
	opt_.cells_per_range = o.cells_per_range;
	opt_.warps_per_block = o.warps_per_block;
	opt_.occupancy = o.occupancy;
	opt_.schedule = o.schedule;
	opt_.agent_lanes = o.agent_lanes;
	return configure();
}

bool Engine::autotune(int trial_steps, EngineOptions* chosen)
{
	if (!sync()) return false;
	if (trial_steps < 1) trial_steps = 1;
	const EngineOptions base = opt_;
	EngineOptions best = opt_;
	float best_ms = 1e30f;
	const bool prof = profile_;
	profile_ = false;
	if (!take_snapshot()) return false;
	bool any_quad = false;
	for (const auto& g : groups_) any_quad |= g.quad_ok;
	const std::vector<int> lanes = any_quad ? std::vector<int>{ 8, 32 } : std::vector<int>{ base.agent_lanes };
	for (int ln : lanes)
	for (float cpr : { 1.0f, 2.0f, 3.0f })
		for (int wpb : { 2, 4 })
			for (float occ : { 1.0f, 0.5f })
				for (int sched : { 0, 1, 2 }) {
					opt_ = base;
					opt_.cells_per_range = cpr; opt_.warps_per_block = wpb; opt_.occupancy = occ; opt_.schedule = sched;
					opt_.agent_lanes = ln;
					if (!configure()) return false;
					if (!restore_snapshot()) return false;
					if (!run_steps(1)) return false;   // graph capture, warm-up
					CK(cudaEventRecord(ev0_, stream_));
					if (!run_steps(trial_steps)) return false;
					CK(cudaEventRecord(ev1_, stream_));
					CK(cudaEventSynchronize(ev1_));
					float ms = 0;
					cudaEventElapsedTime(&ms, ev0_, ev1_);
					int st = 0;
					CK(cudaMemcpy(&st, d_->status, sizeof(int), cudaMemcpyDeviceToHost));
					if (st) {   // a trial overflowed the neighbour capacity: grow it, discard the trial
						CK(cudaMemset(d_->status, 0, sizeof(int)));
						if (st & ST_NEIGHBOUR_OVERFLOW) maxnb_ = grown_capacity(maxnb_);
						continue;
					}
					if (ms < best_ms) { best_ms = ms; best = opt_; }
				}
	opt_ = best;
	if (!configure()) return false;
	if (!restore_snapshot()) return false;
	snap_steps_ = 0;
	CK(cudaStreamSynchronize(stream_));
	snap_valid_ = false;
	profile_ = prof;
	if (chosen) *chosen = best;
	return true;
}

void* Engine::device_positions() const { return d_->pos; }
void* Engine::device_velocities() const { return d_->vel; }

// ------------------------------------------------------------------------
// differentiable form (host)
// ------------------------------------------------------------------------
bool Engine::set_force_params(int scen, const float* p4)
{
	if (!sync()) return false;
	if (scen >= (int)scen_.size()) { err_ = "no scenario " + std::to_string(scen); return false; }
	for (size_t pi = 0; pi < pols_.size(); ++pi) {
		if (scen >= 0 && pol_scen_[pi] != scen) continue;
		PolicyDesc& P = pols_[pi];
		for (int c = 0; c < P.ncost; ++c) {
			CostDesc& C = P.cost[c];
			bool changed = false;
			auto put = [&](int k, float v) { if (!std::isnan(v)) { C.p[k] = v; changed = true; } };
			if (C.kind == K_SOCIALFORCES) { put(1, p4[0]); put(2, p4[1]); }
			else if (C.kind == K_POWERLAW) { put(0, p4[2]); put(1, p4[3]); }
			if (!changed) continue;
			char* dst = (char*)d_->pols + pi * sizeof(PolicyDesc) + offsetof(PolicyDesc, cost) + c * sizeof(CostDesc) +
			            offsetof(CostDesc, p);
			CK(cudaMemcpy(dst, C.p, sizeof(C.p), cudaMemcpyHostToDevice));
		}
	}
	return true;
}

bool Engine::get_force_params(int scen, float* p4)
{
	if (scen < 0 || scen >= (int)scen_.size()) { err_ = "no scenario " + std::to_string(scen); return false; }
	for (int k = 0; k < 4; ++k) p4[k] = NAN;
	for (size_t pi = 0; pi < pols_.size(); ++pi) {
		if (pol_scen_[pi] != scen) continue;
		const PolicyDesc& P = pols_[pi];
		for (int c = 0; c < P.ncost; ++c) {
			const CostDesc& C = P.cost[c];
			if (C.kind == K_SOCIALFORCES && std::isnan(p4[0])) { p4[0] = C.p[1]; p4[1] = C.p[2]; }
			if (C.kind == K_POWERLAW && std::isnan(p4[2])) { p4[2] = C.p[0]; p4[3] = C.p[1]; }
		}
	}
	return true;
}

void Engine::diff_free()
{
	Diff& D = df_;
	void* ptrs[] = { D.s0_pos, D.s0_vel, D.s0_view, D.s0_vwf, D.s0_rng, D.targets, D.ck_pos, D.ck_vel, D.seg_pos,
	                 D.seg_vel, D.seg_acc, D.tape, D.tape_cnt, D.lam_p, D.lam_v, D.lo_p, D.lo_v, D.adj_nb, D.dparams,
	                 D.loss, D.obs_list };
	for (void* p : ptrs)
		if (p) cudaFree(p);
	D = Diff();
}

void Engine::diff_end()
{
	if (stream_) cudaStreamSynchronize(stream_);
	diff_free();
}

bool Engine::diff_begin(int steps, int every, const float* targets, float weight)
{
	if (!sync()) return false;
	diff_free();
	if (steps <= 0 || every <= 0) { err_ = "steps and checkpoint interval must be positive"; return false; }
	if (!pending_.empty() || any_remove_at_goal_) {
		err_ = "the differentiable form needs a fixed agent set (no delayed starts, no removal at the goal)";
		return false;
	}
	for (size_t pi = 0; pi < pols_.size(); ++pi) {
		const PolicyDesc& P = pols_[pi];
		bool ok = P.method == M_GRADIENT;
		for (int c = 0; c < P.ncost; ++c) {
			const int k = P.cost[c].kind;
			ok &= k == K_SOCIALFORCES || k == K_POWERLAW || k == K_GOALREACHING;
		}
		if (!ok) {
			err_ = "the differentiable form supports gradient-method policies made of SocialForcesAvoidance, "
			       "PowerLaw and GoalReachingForce only";
			return false;
		}
	}
	Diff& D = df_;
	const int n = n_;
	D.steps = steps; D.every = std::min(every, steps); D.n = n;
	D.nck = (steps + D.every - 1) / D.every;
	D.weight = weight > 0 ? weight : (float)(1.0 / ((double)steps * std::max(n, 1)));
	const size_t nn = std::max(n, 1);
	if (!dalloc(D.s0_pos, nn, err_) || !dalloc(D.s0_vel, nn, err_) || !dalloc(D.s0_view, nn, err_) ||
	    !dalloc(D.s0_vwf, nn, err_) || !dalloc(D.s0_rng, nn, err_) || !dalloc(D.targets, nn * steps, err_) ||
	    !dalloc(D.ck_pos, nn * D.nck, err_) || !dalloc(D.ck_vel, nn * D.nck, err_) ||
	    !dalloc(D.seg_pos, nn * (D.every + 1), err_) || !dalloc(D.seg_vel, nn * (D.every + 1), err_) ||
	    !dalloc(D.seg_acc, nn * D.every, err_) || !dalloc(D.tape_cnt, nn * D.every, err_) ||
	    !dalloc(D.lam_p, nn, err_) || !dalloc(D.lam_v, nn, err_) || !dalloc(D.lo_p, nn, err_) ||
	    !dalloc(D.lo_v, nn, err_) || !dalloc(D.adj_nb, nn, err_) || !dalloc(D.dparams, 4 * scen_.size(), err_) ||
	    !dalloc(D.loss, 1, err_)) {
		diff_free();
		return false;
	}
	const DevState& S = *d_;
	if (n > 0) {
		CK(cudaMemcpy(D.targets, targets, sizeof(float2) * (size_t)n * steps, cudaMemcpyHostToDevice));
		CK(cudaMemcpy(D.s0_pos, S.pos, sizeof(float2) * n, cudaMemcpyDeviceToDevice));
		CK(cudaMemcpy(D.s0_vel, S.vel, sizeof(float2) * n, cudaMemcpyDeviceToDevice));
		CK(cudaMemcpy(D.s0_view, S.view, sizeof(float2) * n, cudaMemcpyDeviceToDevice));
		CK(cudaMemcpy(D.s0_vwf, S.vwf, sizeof(float2) * n, cudaMemcpyDeviceToDevice));
		CK(cudaMemcpy(D.s0_rng, S.rng, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice));
	}
	D.t0 = time_;
	D.times0 = times_;
	return true;
}

bool Engine::diff_restore_start()
{
	Diff& D = df_;
	const DevState& S = *d_;
	if (D.n > 0) {
		CK(cudaMemcpyAsync(S.pos, D.s0_pos, sizeof(float2) * D.n, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.vel, D.s0_vel, sizeof(float2) * D.n, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.view, D.s0_view, sizeof(float2) * D.n, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.vwf, D.s0_vwf, sizeof(float2) * D.n, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.rng, D.s0_rng, sizeof(uint32_t) * D.n, cudaMemcpyDeviceToDevice, stream_));
	}
	time_ = D.t0;
	times_ = D.times0;
	return true;
}

// Waits for the stream; true when no device condition was raised.  A
// neighbour-capacity overflow is reported through *overflow (the caller
// re-runs with a grown capacity).
bool Engine::diff_check_status()
{
	CK(cudaStreamSynchronize(stream_));
	int st = 0;
	CK(cudaMemcpy(&st, d_->status, sizeof(int), cudaMemcpyDeviceToHost));
	if (st == 0) return true;
	CK(cudaMemset(d_->status, 0, sizeof(int)));
	if ((st & ST_NEIGHBOUR_OVERFLOW) && maxnb_ < 3072) {
		maxnb_ = grown_capacity(maxnb_);
		invalidate_graph();
		err_ = "overflow";
		return false;
	}
	if (st & ST_NEIGHBOUR_OVERFLOW) err_ = "a neighbour list is longer than " + std::to_string(maxnb_) + " entries";
	else if (st & ST_GRID_OVERFLOW) err_ = "non-finite agent positions";
	else err_ = "device status " + std::to_string(st);
	return false;
}

bool Engine::diff_forward(double* loss)
{
	Diff& D = df_;
	if (D.steps == 0) { err_ = "no differentiable episode (call diff_begin first)"; return false; }
	if (!sync()) return false;
	D.forward_done = false;
	const int n = D.n;
	// the last segment is recorded as it runs (lists, states, accelerations),
	// so that the backward pass starts reversing without recomputing it
	const int last0 = (D.nck - 1) * D.every;
	DevState& S = *d_;
	for (;;) {
		if (!diff_restore_start()) return false;
		if (configured_maxnb_ != maxnb_ && !configure()) return false;
		if (!diff_alloc_tape()) return false;
		CK(cudaMemsetAsync(D.loss, 0, sizeof(double), stream_));
		for (int t = 0; t < D.steps; ++t) {
			if (t % D.every == 0 && n > 0) {
				const size_t c = (size_t)(t / D.every) * n;
				CK(cudaMemcpyAsync(D.ck_pos + c, S.pos, sizeof(float2) * n, cudaMemcpyDeviceToDevice, stream_));
				CK(cudaMemcpyAsync(D.ck_vel + c, S.vel, sizeof(float2) * n, cudaMemcpyDeviceToDevice, stream_));
			}
			if (t >= last0 && n > 0) {
				const int st = t - last0;
				CK(cudaMemcpyAsync(D.seg_pos + (size_t)st * n, S.pos, sizeof(float2) * n, cudaMemcpyDeviceToDevice,
				                   stream_));
				CK(cudaMemcpyAsync(D.seg_vel + (size_t)st * n, S.vel, sizeof(float2) * n, cudaMemcpyDeviceToDevice,
				                   stream_));
				S.tape_list = D.tape + (size_t)st * n * maxnb_;
				S.tape_cnt = D.tape_cnt + (size_t)st * n;
				S.tape_acc = D.seg_acc + (size_t)st * n;
				steps_pending_ = true;
				enqueue_step();
				S.tape_list = nullptr; S.tape_cnt = nullptr; S.tape_acc = nullptr;
				time_ += sc_.dt;
				for (size_t k = 0; k < times_.size(); ++k) times_[k] += scen_[k].dt;
			} else if (!run_steps(1)) {
				return false;
			}
			if (n > 0) k_loss<<<(n + 255) / 256, 256, 0, stream_>>>(S, D.targets + (size_t)t * n, D.weight, D.loss);
		}
		if (n > 0)
			CK(cudaMemcpyAsync(D.seg_pos + (size_t)(D.steps - last0) * n, S.pos, sizeof(float2) * n,
			                   cudaMemcpyDeviceToDevice, stream_));
		CK(cudaGetLastError());
		if (diff_check_status()) break;
		if (err_ != "overflow") return false;
	}
	D.forward_done = true;
	if (loss) CK(cudaMemcpy(loss, D.loss, sizeof(double), cudaMemcpyDeviceToHost));
	return true;
}

bool Engine::diff_alloc_tape()
{
	Diff& D = df_;
	if (D.tape && D.tape_nb == maxnb_) return true;
	if (D.tape) cudaFree(D.tape);
	D.tape = nullptr;
	D.tape_nb = maxnb_;
	return dalloc(D.tape, (size_t)std::max(D.n, 1) * D.every * maxnb_, err_);
}

bool Engine::diff_backward(float* dparams, float* dpos0, float* dvel0)
{
	Diff& D = df_;
	if (!D.forward_done) { err_ = "diff_backward needs a completed diff_forward"; return false; }
	if (!diff_alloc_tape()) return false;
	DevState& S = *d_;
	const int n = D.n;
	const size_t nb2 = sizeof(float2) * std::max(n, 1);
	CK(cudaMemsetAsync(D.lam_p, 0, nb2, stream_));
	CK(cudaMemsetAsync(D.lam_v, 0, nb2, stream_));
	CK(cudaMemsetAsync(D.dparams, 0, sizeof(float) * 4 * scen_.size(), stream_));
	const int adj_blocks = std::max(1, std::min((n + 3) / 4, num_sms_ * 5));
	// per-warp obstacle lists of k_adjoint, at the capacity the step uses
	// (configure sets it; at most num_sms * 5 blocks of 4 warps)
	if (!edges_.empty() && D.obs_cap != S.max_obs) {
		if (D.obs_list) cudaFree(D.obs_list);
		D.obs_list = nullptr;
		D.obs_cap = 0;
		if (S.max_obs <= 0) { err_ = "obstacle list capacity not configured"; return false; }
		if (!dalloc(D.obs_list, (size_t)num_sms_ * 5 * 4 * S.max_obs, err_)) return false;
		D.obs_cap = S.max_obs;
	}
	for (int c = D.nck - 1; c >= 0 && n > 0; --c) {
		const int t0 = c * D.every, m = std::min(D.every, D.steps - t0);
		// recompute the segment from its checkpoint, recording lists and states
		// (the forward pass recorded the last one)
		CK(cudaMemcpyAsync(S.pos, D.ck_pos + (size_t)c * n, sizeof(float2) * n, cudaMemcpyDeviceToDevice, stream_));
		CK(cudaMemcpyAsync(S.vel, D.ck_vel + (size_t)c * n, sizeof(float2) * n, cudaMemcpyDeviceToDevice, stream_));
		for (int s = 0; s < m && c < D.nck - 1; ++s) {
			CK(cudaMemcpyAsync(D.seg_pos + (size_t)s * n, S.pos, sizeof(float2) * n, cudaMemcpyDeviceToDevice, stream_));
			CK(cudaMemcpyAsync(D.seg_vel + (size_t)s * n, S.vel, sizeof(float2) * n, cudaMemcpyDeviceToDevice, stream_));
			S.tape_list = D.tape + (size_t)s * n * maxnb_;
			S.tape_cnt = D.tape_cnt + (size_t)s * n;
			S.tape_acc = D.seg_acc + (size_t)s * n;
			enqueue_step();
			S.tape_list = nullptr; S.tape_cnt = nullptr; S.tape_acc = nullptr;
		}
		if (c < D.nck - 1)
			CK(cudaMemcpyAsync(D.seg_pos + (size_t)m * n, S.pos, sizeof(float2) * n, cudaMemcpyDeviceToDevice,
			                   stream_));
		// reverse the segment
		for (int s = m - 1; s >= 0; --s) {
			k_inject<<<(n + 255) / 256, 256, 0, stream_>>>(n, D.seg_pos + (size_t)(s + 1) * n,
			                                               D.targets + (size_t)(t0 + s) * n, D.weight, D.lam_p,
			                                               D.lam_v, D.lo_p, D.lo_v);
			CK(cudaMemsetAsync(D.lam_p, 0, nb2, stream_));
			CK(cudaMemsetAsync(D.lam_v, 0, nb2, stream_));
			DevState A = S;
			A.tape_list = D.tape + (size_t)s * n * maxnb_;
			A.tape_cnt = D.tape_cnt + (size_t)s * n;
			A.tape_acc = D.seg_acc + (size_t)s * n;
			A.a_pos = D.seg_pos + (size_t)s * n;
			A.a_vel = D.seg_vel + (size_t)s * n;
			A.lam_out_p = D.lo_p; A.lam_out_v = D.lo_v;
			A.lam_in_p = D.lam_p; A.lam_in_v = D.lam_v;
			A.dparams = D.dparams;
			A.adj_nb = D.adj_nb;
			A.obs_list = D.obs_list;   // k_adjoint warps (at most num_sms * 5 blocks of 4)
			k_adj_prep<<<(n + 255) / 256, 256, 0, stream_>>>(A);
			if (edges_.empty()) k_adjoint<false><<<adj_blocks, 128, 0, stream_>>>(A);
			else k_adjoint<true><<<adj_blocks, 128, 0, stream_>>>(A);
		}
	}
	CK(cudaGetLastError());
	if (!diff_check_status()) {
		if (err_ == "overflow") err_ = "neighbour lists of the recomputed segment outgrew the capacity";
		return false;
	}
	if (dparams) CK(cudaMemcpy(dparams, D.dparams, sizeof(float) * 4 * scen_.size(), cudaMemcpyDeviceToHost));
	if (dpos0 && n > 0) CK(cudaMemcpy(dpos0, D.lam_p, sizeof(float2) * n, cudaMemcpyDeviceToHost));
	if (dvel0 && n > 0) CK(cudaMemcpy(dvel0, D.lam_v, sizeof(float2) * n, cudaMemcpyDeviceToHost));
	if (!diff_restore_start()) return false;
	CK(cudaStreamSynchronize(stream_));
	return true;
}

Engine::~Engine()
{
	if (stream_) cudaStreamSynchronize(stream_);
	invalidate_graph();
	record_stop();
	for (cudaEvent_t e : rec_ev_)
		if (e) cudaEventDestroy(e);
	diff_free();
	if (io_host_) cudaFreeHost(io_host_);
	if (status_host_) cudaFreeHost(status_host_);
	if (d_) {
		DevState& S = *d_;
		void* ptrs[] = { S.pos, S.vel, S.goal, S.view, S.vwf, S.pref, S.prm, S.pol, S.id, S.rng, S.sP, S.sV, S.sB, S.sE,
		                 S.sSlot, S.sId, S.cell, S.cnt, S.start, S.blocksum, S.grid, S.bbox, S.status,
		                 (void*)S.pols, (void*)S.table, (void*)S.lcgpow, S.scratch, S.dump_ids, S.dump_cnt, S.dump_d2, S.slot_of_id, S.io,
		                 S.agent_scen, S.cell_base, scen_dev_, S.obs_list, S.work,
		                 snap_pos_, snap_vel_, snap_view_, snap_vwf_, snap_rng_ };
		for (void* p : ptrs)
			if (p) cudaFree(p);
		delete d_;
	}
	for (cudaEvent_t e : { pa0_, pa1_, ps0_, ps1_ })
		if (e) cudaEventDestroy(e);
	if (scen_order_dev_) cudaFree(scen_order_dev_);
	if (edges_dev_) cudaFree(edges_dev_);
	if (og_start_dev_) cudaFree(og_start_dev_);
	if (og_items_dev_) cudaFree(og_items_dev_);
	if (og_ecell_dev_) cudaFree(og_ecell_dev_);
	if (counters_) cudaFree(counters_);
	if (ev0_) cudaEventDestroy(ev0_);
	if (ev1_) cudaEventDestroy(ev1_);
	if (stream_) cudaStreamDestroy(stream_);
}

}  // namespace umans
