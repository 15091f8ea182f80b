// grid build: bounding box, cell histogram, scan, counting-sort scatter,
// the one-launch cooperative build and the small-world build
//
// Device code of the step engine, part of engine.cu's translation unit:
// included once, from engine.cu, after DevState; uses its helpers.
#pragma once

namespace umans {

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

// grid over the box (x0, y0) + (ex, ey): the cell size range /
// cells_per_range, doubled until the grid has at most max_cells cells
__device__ __forceinline__ GridParams grid_of_box(const DevState& S, const ScenDesc& sd, float x0, float y0, float ex,
                                                  float ey, int max_cells)
{
	if (!isfinite(x0) || !isfinite(y0) || !isfinite(ex) || !isfinite(ey)) {
		atomicOr(S.status, ST_GRID_OVERFLOW);
		x0 = y0 = 0; ex = ey = 1;
	}
	float cs = sd.max_range / S.cells_per_range;
	if (!(cs >= 1e-3f)) cs = 1e-3f;
	// +2 per axis: nx, ny below come from float divisions that may round up
	while (((double)ex / cs + 2.0) * ((double)ey / cs + 2.0) > (double)max_cells) cs *= 2.0f;
	GridParams g;
	g.x0 = x0; g.y0 = y0; g.cs = cs; g.inv_cs = 1.0f / cs;
	g.nx = (int)(ex / cs) + 1; g.ny = (int)(ey / cs) + 1;
	g.ncells = g.nx * g.ny; g.pad = 0;
	return g;
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
	const GridParams g = grid_of_box(S, sd, x0, y0, ex, ey, sd.max_cells);
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

// the cell-sorted copies of agent i (position p) at index t, with its
// preferred velocity
__device__ __forceinline__ void scatter_to(const DevState& S, int i, int t, float2 p)
{
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
	scatter_to(S, i, t, S.pos[i]);
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
__device__ __forceinline__ void build_small(const DevState& S)
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
__global__ void __launch_bounds__(1024) k_build_small(DevState S)
{
	build_small(S);
}

// build_small for k_small_steps, with the bounding box, the histogram and
// the scan in shared memory: global memory only gives the agents' state and
// takes the cell-sorted copies, the cell starts and the grid parameters.
// The grid has at most SMALL_SMEM_CELLS cells (the cell size is doubled
// until it fits, as for any cell cap; no neighbour list depends on it).
constexpr int SMALL_SMEM_CELLS = 4096;
struct SmallGrid {
	int cnt[SMALL_SMEM_CELLS];
	int start[SMALL_SMEM_CELLS + 1];
	unsigned box[4];
	int tot[32];
	GridParams g;
};
__device__ __forceinline__ void build_small_smem(const DevState& S, SmallGrid& B)
{
	const int n = S.n, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
	const ScenDesc& sd = S.scen[0];
	const int world = sd.world;
	if (world != W_TORIC) {
		unsigned a = f2o(FLT_MAX), b = a, c = f2o(-FLT_MAX), d = c;
		for (int i = tid; i < n; i += nt) {
			const float2 p = S.pos[i];
			a = min(a, f2o(p.x)); b = min(b, f2o(p.y));
			c = max(c, f2o(p.x)); d = max(d, f2o(p.y));
		}
		a = __reduce_min_sync(0xffffffffu, a); b = __reduce_min_sync(0xffffffffu, b);
		c = __reduce_max_sync(0xffffffffu, c); d = __reduce_max_sync(0xffffffffu, d);
		if (tid < 4) B.box[tid] = tid < 2 ? f2o(FLT_MAX) : f2o(-FLT_MAX);
		__syncthreads();
		if (lane == 0) {
			atomicMin(&B.box[0], a); atomicMin(&B.box[1], b);
			atomicMax(&B.box[2], c); atomicMax(&B.box[3], d);
		}
		__syncthreads();
	}
	if (tid == 0) {
		// the box as grid_params takes it
		float x0, y0, ex, ey;
		if (world == W_TORIC) {
			x0 = -0.5f * sd.width; y0 = -0.5f * sd.height; ex = sd.width; ey = sd.height;
		} else {
			x0 = o2f(B.box[0]); y0 = o2f(B.box[1]);
			ex = o2f(B.box[2]) - x0; ey = o2f(B.box[3]) - y0;
			if (sd.n == 0) { x0 = y0 = 0; ex = ey = 1; }
		}
		const GridParams g = grid_of_box(S, sd, x0, y0, ex, ey, min(sd.max_cells, SMALL_SMEM_CELLS));
		S.grid[0] = g;
		S.cell_base[0] = 0;
		S.cell_base[1] = g.ncells;
		B.g = g;
	}
	__syncthreads();
	const GridParams g = B.g;
	const int nc = g.ncells;
	for (int c = tid; c < nc; c += nt) B.cnt[c] = 0;
	__syncthreads();
	for (int i = tid; i < n; i += nt) {
		const float2 p = S.pos[i];
		atomicAdd(&B.cnt[cell_coord(p.y, g.y0, g.inv_cs, g.ny) * g.nx + cell_coord(p.x, g.x0, g.inv_cs, g.nx)], 1);
	}
	__syncthreads();
	// exclusive scan: a run of cells per thread, then the threads' sums
	const int per = (nc + nt - 1) / nt;
	const int c0 = min(nc, tid * per), c1 = min(nc, c0 + per);
	int local = 0;
	for (int c = c0; c < c1; ++c) local += B.cnt[c];
	int incl = local;
	for (int o = 1; o < 32; o <<= 1) {
		const int v = __shfl_up_sync(0xffffffffu, incl, o);
		if (lane >= o) incl += v;
	}
	if (lane == 31) B.tot[wid] = incl;
	__syncthreads();
	if (wid == 0) {
		const int v = lane < nw ? B.tot[lane] : 0;
		int w = v;
		for (int o = 1; o < 32; o <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, w, o);
			if (lane >= o) w += u;
		}
		B.tot[lane] = w - v;
	}
	__syncthreads();
	int run = B.tot[wid] + incl - local;
	for (int c = c0; c < c1; ++c) {
		B.start[c] = run;
		S.start[c] = run;
		run += B.cnt[c];
	}
	if (tid == 0) S.start[nc] = n;
	__syncthreads();
	// the scatter fills each cell from its top down
	for (int i = tid; i < n; i += nt) {
		const float2 p = S.pos[i];
		const int c = cell_coord(p.y, g.y0, g.inv_cs, g.ny) * g.nx + cell_coord(p.x, g.x0, g.inv_cs, g.nx);
		const int t = B.start[c] + atomicSub(&B.cnt[c], 1) - 1;
		scatter_to(S, i, t, p);
	}
}

}  // namespace umans
