// GB300 step engine: the per-step agent update of WorldBase::DoStep
// (src/Engine/core/worldBase.cpp:79-128) as a short kernel sequence.
//
// Grid build (grid.cuh), into cell-sorted copies of position / velocity /
// preferred velocity / radius, the preferred velocity computed on the way
// (agent.cpp:52-59):
//   k_grid_coop         toric worlds: histogram, scan and scatter in one
//                       cooperative launch (grid parameters fixed once)
//   k_build_small       one block for a small single-scenario world
//   k_bbox / k_grid,    otherwise: bounding box and grid parameters
//   k_count, k_scan_*,  (infinite worlds), per-cell histogram, exclusive
//   k_scatter           scan, counting-sort scatter
// Agent update, one launch per kernel group (scenarios grouped by the
// specialisation their policies allow), agents in cell order:
//   k_force_quad        force-only policies, four agents per warp
//                       (quad_kernels.cuh)
//   k_agent<MODE>       one warp per agent: general, force-only with
//                       obstacles, ORCA-only, Karamouzas-sampling
//                       (agent_kernels.cuh)
// each doing the neighbour query (kd-tree radius search semantics,
// AgentKDTree.cpp:35-59, worldToric.cpp:32-79; neighbours.cuh), contact
// forces (policy.cpp:107-141), the velocity optimisation (policy.cpp:43-105;
// evaluate.cuh, agent_step.cuh) and the integration with the toric wrap
// (agent.cpp:71-93, worldToric.cpp:81-108).
//
// Phases 2-6 of DoStep only read state that earlier phases finished and only
// write per-agent state, so they fuse into one kernel: every neighbour read
// goes to the cell-sorted copies made by the scatter, every write to the
// agent's own slot.  adjoint_kernels.cuh holds the differentiable form's
// backward kernels, agent_io.cuh the AgentData exchange, math_checks.cuh the
// device math tables and their test entry points; this file the host side.
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

}  // namespace umans

#include "grid.cuh"
#include "neighbours.cuh"
#include "evaluate.cuh"
#include "agent_step.cuh"
#include "quad_kernels.cuh"
#include "agent_kernels.cuh"
#include "math_checks.cuh"
#include "adjoint_kernels.cuh"
#include "agent_io.cuh"

namespace umans {

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
	small_steps_occupancy();
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

// k_small_steps: the lists, then (16-byte aligned) 2 * maxnb float4 of
// lines per warp
static size_t small_steps_smem(int warps_per_block, int maxnb, int mode)
{
	return agent_smem(warps_per_block, maxnb, mode) + (size_t)warps_per_block * 2 * maxnb * sizeof(float4) + 16;
}
static constexpr size_t SMALL_STEPS_SMEM = 160 * 1024;   // dynamic shared memory per block, at most (with the static 33 KB, below the 227 KB limit)

// k_small_steps takes a small world whose one kernel group runs k_agent
// (modes 0, 2, 3) and whose steps need no host work in between (no
// trajectory output, profiling or tape).  Blocks of 4 warps (8 above 512
// agents), as many as give every agent its own warp, at most as many as are
// resident at once and as the line scratch covers; 0 blocks when the steps
// of a call cannot run in one launch.
void Engine::small_steps_shape(int* blocks, int* threads) const
{
	*blocks = 0;
	*threads = 0;
	if (!opt_.multi_step || profile_ || n_ < 1 || !small_world() || groups_.size() != 1 || d_->tape_list) return;
	const KGroup& g = groups_[0];
	if (g.quad || g.mode == 1) return;
	const int m = g.mode == 2 ? 2 : (g.mode == 3 ? 3 : 0);
	const int wpb = n_ <= 512 ? 4 : 8;
	const size_t smem = small_steps_smem(wpb, maxnb_, g.mode);
	if (smem > SMALL_STEPS_SMEM) return;
	const int resident = small_steps_resident_[m][wpb == 4 ? 0 : 1];
	if (resident < 1) return;
	int nb = (n_ + wpb - 1) / wpb;
	nb = std::min(nb, resident * num_sms_);
	nb = (int)std::min<long long>(nb, (long long)g.blocks * opt_.warps_per_block / wpb);   // line scratch
	if (nb < 1) return;
	*blocks = nb;
	*threads = wpb * 32;
}

bool Engine::launch_small_steps(int nsteps, int blocks, int threads)
{
	const KGroup& g = groups_[0];
	DevState S = *d_;
	S.n = n_;
	S.maxnb = maxnb_;
	S.counters = nullptr;
	S.t_begin = 0;
	S.t_end = n_;
	S.total_warps = blocks * threads / 32;
	S.sched = 0;
	S.scratch = d_->scratch + g.scratch_off;
	S.obs_list = d_->obs_list + g.obs_off;
	const size_t smem = small_steps_smem(threads / 32, maxnb_, g.mode);
	const int m = g.mode == 2 ? 2 : (g.mode == 3 ? 3 : 0);
	void (*fn)(DevState, int) = m == 2 ? k_small_steps<2> : (m == 3 ? k_small_steps<3> : k_small_steps<0>);
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3((unsigned)blocks);
	cfg.blockDim = dim3((unsigned)threads);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream_;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeCooperative;
	attr[0].val.cooperative = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	CK(cudaLaunchKernelEx(&cfg, fn, S, nsteps));
	return true;
}

// Blocks of k_small_steps resident per SM for the current neighbour
// capacity (by mode, 4 and 8 warps per block; 0 leaves the mode on the
// graph path); configure() refreshes them.
void Engine::small_steps_occupancy()
{
	const int modes[3] = {0, 2, 3};
	for (int m : modes) {
		void (*fn)(DevState, int) = m == 2 ? k_small_steps<2> : (m == 3 ? k_small_steps<3> : k_small_steps<0>);
		// the kernel's static shared memory (build_small_smem's grid) counts
		// against the 48 KB default too: allow the whole budget
		const bool allowed =
		    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMALL_STEPS_SMEM) == cudaSuccess;
		if (!allowed) cudaGetLastError();
		for (int k = 0; k < 2; ++k) {
			const int wpb = k == 0 ? 4 : 8;
			int per_sm = 0;
			const size_t smem = small_steps_smem(wpb, maxnb_, m);
			if (!allowed || smem > SMALL_STEPS_SMEM ||
			    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, wpb * 32, smem) != cudaSuccess) {
				cudaGetLastError();
				per_sm = 0;
			}
			small_steps_resident_[m][k] = per_sm;
		}
	}
}

bool Engine::set_multi_step(bool on)
{
	if (!sync()) return false;
	opt_.multi_step = on;
	return true;
}

int Engine::kernels_per_step() const
{
	int sblocks = 0, sthreads = 0;
	small_steps_shape(&sblocks, &sthreads);
	if (sblocks > 0) return 1;
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
	int sblocks = 0, sthreads = 0;
	if (!record) small_steps_shape(&sblocks, &sthreads);
	if (sblocks > 0) {
		if (!launch_small_steps(nsteps, sblocks, sthreads)) return false;
		for (int s = 0; s < nsteps; ++s) {
			time_ += sc_.dt;
			for (size_t k = 0; k < times_.size(); ++k) times_[k] += scen_[k].dt;
		}
		return true;
	}
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
