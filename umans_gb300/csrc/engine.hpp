// One simulation on one GPU: the GB300 replacement of WorldBase::DoStep
// (src/Engine/core/worldBase.cpp:79-128) behind the reference's simulation
// interface (CrowdSimulator / WorldBase / Agent, src/Engine/core/).
#pragma once
#include <atomic>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "model.hpp"
#include "recorder.hpp"
#include "scenario.hpp"

namespace umans {

struct DevState;   // device pointers (engine.cu)

// device evaluation of the reference-exact expf (refmath.hpp), for tests
bool debug_ref_expf(const float* x, float* y, int n, size_t* exceptions, std::string& err);
// the short exponential against the table-backed one over float bit patterns
// [first, first + count): out[0] answered, out[1] differing, out[2] listed
bool debug_expf_check(uint32_t first, uint32_t count, unsigned long long* out, float* band, std::string& err);
bool debug_ref_sincosf(const float* x, float* s, float* c, int n, size_t* exceptions, std::string& err);
bool set_device_sincos(std::string& err);
// device evaluation of (float)((double)a*b - (double)c*d) (devmath.cuh), for tests
bool debug_prod_diff(const float* abcd, float* y, int n, std::string& err);

struct EngineOptions {
	int max_neighbours = 0;        // 0: chosen from the initial state
	float cells_per_range = 2.0f;  // grid cell size = range / cells_per_range
	int warps_per_block = 4;
	float occupancy = 1.0f;   // fraction of the resident blocks per SM that the agent kernel launches
	int schedule = 0;         // agents to warps: 0 interleaved, 1 contiguous blocks, 2 work list of agent tiles
	int agent_lanes = 8;      // lanes per agent in the force-only groups that allow 8 (else 32)
	bool use_graph = true;
	bool multi_step = true;   // small worlds: the steps of one call in one launch (k_small_steps)
};

class Engine {
public:
	static Engine* create(const std::string& xml, std::string& err, const EngineOptions& opt = EngineOptions());
	// several independent scenarios stepped together (agents concatenated,
	// scenario k at list slots [offset(k), offset(k+1)))
	static Engine* create_batch(const std::vector<std::string>& xmls, std::string& err,
	                            const EngineOptions& opt = EngineOptions());
	int num_scenarios() const { return (int)scen_.size(); }
	int scenario_offset(int k) const { return k < (int)scen_.size() ? scen_[k].agent_off : n_; }
	~Engine();

	// Enqueues n steps on the engine's stream; returns false on a host-side
	// error.  Device-side errors are reported by sync().
	bool step(int n);
	bool sync();

	int num_agents() const { return n_; }
	double time() const { return time_; }
	float dt() const { return sc_.dt; }
	float end_time() const { return sc_.end_time; }
	const std::string& error() const { return err_; }
	cudaStream_t stream() const { return stream_; }
	int max_neighbours() const { return maxnb_; }

	// host <-> device state, list order (the reference's agents_ order)
	bool get_state(int* ids, float* pos, float* vel, float* view, float* pref = nullptr, float* goal = nullptr);
	bool set_state(const float* pos, const float* vel, const float* view);   // all agents, list order
	bool set_agent_by_id(int id, float px, float py, float vx, float vy, float wx, float wy);
	// AgentData records (include/umans_gb300.h), one bulk copy each way
	bool get_agent_data(void* out);
	bool set_agent_data(const void* in, int m);
	bool set_goal(int id, float x, float y);
	bool add_agent(float x, float y, float radius, float pref, float maxs, float maxacc, int policy_id,
	               int desired_id, int* out_id);
	bool remove_agent(int id);

	// neighbour lists the next step would use: ids and PhantomAgent distSqr,
	// `cap` entries per agent; counts[i] = full list length.
	bool neighbours(int cap, int* ids, float* d2, int* counts);

	// times the launch-shape candidates from the current state (restored
	// afterwards) and keeps the fastest
	bool autotune(int trial_steps, EngineOptions* chosen);
	// applies a launch shape (the fields autotune chooses); results do not depend on it
	bool set_launch(const EngineOptions& o);
	// small worlds: every step of a call in one launch (on by default), or
	// one graph launch per step; results do not depend on it
	bool set_multi_step(bool on);
	const EngineOptions& options() const { return opt_; }

	// device pointers of the raw state for callers that keep data on the GPU
	void* device_positions() const;
	void* device_velocities() const;

	// timing of the step kernels (ms, averaged over the last step() call)
	float last_agent_kernel_ms() const { return agent_ms_; }
	bool time_kernels = false;

	// Profiling mode: every step is launched without the graph, with CUDA
	// events on the engine's stream around the step and around k_agent;
	// the elapsed times accumulate until reset.
	void set_profile(bool on);
	// counters of the last profiled steps (see DevState::counters)
	bool profile_counters(unsigned long long* out, int n);
	void profile_totals(double* agent_ms, double* step_ms, int* steps, double* grid_ms) const
	{ *agent_ms = prof_agent_ms_; *step_ms = prof_step_ms_; *steps = prof_steps_; *grid_ms = prof_grid_ms_; }
	int kernels_per_step() const;
	bool small_world() const;   // one-block grid build (k_build_small)
	// launch shape of k_small_steps for the current state (0 blocks when the
	// steps of a call cannot run in one launch)
	void small_steps_shape(int* blocks, int* threads) const;

	// ---- differentiable form ------------------------------------------
	// Episode: `steps` steps from the current state (recorded as the
	// episode's start), loss L = weight * sum_t sum_i |p_i(t) - target_i(t)|^2
	// over t = 1..steps (targets: steps x n x 2 floats, list order; weight
	// <= 0 means 1 / (steps * n)).  Checkpoints every `every` steps; the
	// backward pass recomputes each segment from its checkpoint with the
	// neighbour lists recorded and reverses it with k_adjoint.  Every policy
	// must use the gradient method with SocialForcesAvoidance, PowerLaw and
	// GoalReachingForce costs only; agents are neither added nor removed.
	bool diff_begin(int steps, int every, const float* targets, float weight);
	bool diff_forward(double* loss);   // from the episode's start state
	// dparams: [num_scenarios x 4] dL/d(V0, sigma, k, tau0); dpos0/dvel0:
	// [n x 2] dL/d(initial positions, velocities) (each may be null).  The
	// state is then the episode's start state again.
	bool diff_backward(float* dparams, float* dpos0, float* dvel0);
	void diff_end();
	// (V0, sigma) of the SocialForcesAvoidance costs and (k, tau0) of the
	// PowerLaw costs of scenario `scen` (all scenarios when scen < 0); NaN
	// entries are left unchanged.  get: NaN where the scenario has no such cost.
	bool set_force_params(int scen, const float* p4);
	bool get_force_params(int scen, float* p4);

	// ---- trajectory output -------------------------------------------
	// Positions of every step are kept in a device ring of `ring_steps`
	// steps and written (TrajWriter formats) when the ring is full, on
	// flush and on stop; population changes flush first.
	bool record_start(const std::string& dir, int ring_steps, int format);
	bool record_flush();   // everything recorded so far written to disk
	bool record_stop();
	int diff_kernels_forward_per_step() const { return kernels_per_step() + 1; }

private:
	Engine() = default;
	bool init(const std::vector<std::string>& xmls, const EngineOptions& opt);
	bool upload_all();
	bool alloc(int cap);
	bool build_tables();
	bool choose_maxnb();
	bool configure();
	bool run_steps(int n, bool record = false);
	bool take_snapshot();
	bool restore_snapshot();
	void enqueue_step();
	void enqueue_grid(const DevState& S);
	bool ensure_static_grid();
	cudaError_t launch_grid_coop(const DevState& S);
	void probe_grid_coop();
	bool launch_small_steps(int nsteps, int blocks, int threads);
	void small_steps_occupancy();
	int small_steps_resident_[4][2] = {};   // per mode: blocks per SM at 4 and 8 warps per block
	int coop_state_ = 0;        // one-launch grid build: 0 untried, 1 usable, -1 not capturable
	int coop_blocks_max_ = 1;
	bool toric_only_ = false;          // every scenario's world is toric: the grid is fixed
	bool static_grid_ready_ = false;   // its parameters are on the device
	int static_cells_ = 0;             // its cell count
	bool capture_graph();
	void invalidate_graph();
	bool apply_pending_agents();
	struct AgentLists;
	void take_lists(AgentLists& L);
	void append_agent(const AgentLists& L, int i);
	void append_new_agent(const AgentInit& a);
	double scen_time(int k) const;
	bool agents_due() const;
	bool finish_list_change();
	bool remove_at_goal();
	bool download_mutable();

	Scenario sc_;                    // scenario 0 (single-simulation API)
	std::vector<Scenario> scs_;
	std::vector<ScenDesc> scen_;
	ScenDesc* scen_dev_ = nullptr;
	std::vector<PolicyDesc> pols_;   // all scenarios' policies, concatenated
	std::vector<int> agent_scen_;
	std::vector<double> times_, snap_times_;
	EngineOptions opt_;
	std::string err_;
	int n_ = 0, cap_ = 0;
	double time_ = 0;
	int maxnb_ = 0, configured_maxnb_ = -1;
	int num_sms_ = 0, agent_blocks_ = 0, mode_ = 0;
	int next_unused_id_ = 0;
	bool any_remove_at_goal_ = false;
	float agent_ms_ = 0;

	// host mirror, list order
	std::vector<int> id_, pol_;
	std::vector<float2> pos_, vel_, goal_, view_, vwf_;
	std::vector<float4> prm_;   // radius, pref speed, max speed, max acceleration
	std::vector<uint32_t> rng_;
	std::vector<unsigned char> remove_;
	std::unordered_map<int, int> slot_of_;
	std::vector<AgentInit> pending_;   // start_time > now, sorted by start_time

	DevState* d_ = nullptr;
	cudaStream_t stream_ = nullptr;
	cudaGraph_t graph_ = nullptr;
	cudaGraphExec_t graph_exec_ = nullptr;
	bool graph_valid_ = false;
	cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
	cudaEvent_t pa0_ = nullptr, pa1_ = nullptr, ps0_ = nullptr, ps1_ = nullptr;
	bool profile_ = false;
	unsigned long long* counters_ = nullptr;   // [3], device
	// batch snapshot for re-running a batch after a capacity overflow
	float2 *snap_pos_ = nullptr, *snap_vel_ = nullptr, *snap_view_ = nullptr, *snap_vwf_ = nullptr;
	uint32_t* snap_rng_ = nullptr;
	int snap_cap_ = 0, snap_steps_ = 0;
	bool snap_valid_ = false;
	bool steps_pending_ = false;   // steps enqueued whose status has not been read
	double snap_time_ = 0;
	double prof_agent_ms_ = 0, prof_step_ms_ = 0, prof_grid_ms_ = 0;
	int prof_steps_ = 0;
	std::vector<int> pol_scen_;   // scenario of each policy
	bool need_trig_ = false;      // a policy samples random rotations (build_tables)
	// k_agent launches: one per kernel group (scenarios ordered by group in
	// cell space)
	struct KGroup {
		int mode;          // k_agent specialisation
		int j0, j1;        // positions in scen_order_
		int blocks;
		size_t scratch_off, obs_off;
		bool obst = false;   // a scenario of the group has obstacle edges
		bool quad_ok = false;   // k_force_quad allowed: force-only, no obstacle edges, <= 1 neighbour cost per policy
		bool quad = false;      // k_force_quad chosen (quad_ok and EngineOptions::agent_lanes == 8)
		bool samp = false;   // a force-only group with a policy of the sampling or global method
		bool sf_only = false;   // every neighbour cost of the group is SocialForces
	};
	std::vector<KGroup> groups_;
	std::vector<int> scen_order_;
	int* scen_order_dev_ = nullptr;
	std::vector<float4> edges_;      // obstacle edges of all scenarios
	float4* edges_dev_ = nullptr;
	// edge grids (ScenDesc::og_*): per scenario cell starts, items (global
	// edge index, cell x), and each edge's cell range (x0, y0, x1, y1)
	std::vector<int> og_start_;
	std::vector<int2> og_items_;
	std::vector<int4> og_ecell_;
	int* og_start_dev_ = nullptr;
	int2* og_items_dev_ = nullptr;
	int4* og_ecell_dev_ = nullptr;
	void build_edge_grids();
	AgentRecord* io_host_ = nullptr;   // page-locked staging for AgentData exchange
	int* status_host_ = nullptr;       // page-locked copy of the device status word
	size_t io_host_cap_ = 0;
	bool stage(size_t records);

	// differentiable form (device buffers; see diff_begin)
	struct Diff {
		int steps = 0, every = 0, nck = 0, n = 0, tape_nb = 0;
		float weight = 0;
		bool forward_done = false;
		double t0 = 0;
		std::vector<double> times0;
		float2 *s0_pos = nullptr, *s0_vel = nullptr, *s0_view = nullptr, *s0_vwf = nullptr;
		uint32_t* s0_rng = nullptr;
		float2* targets = nullptr;                   // steps x n
		float2 *ck_pos = nullptr, *ck_vel = nullptr;   // nck x n
		float2 *seg_pos = nullptr, *seg_vel = nullptr, *seg_acc = nullptr;   // (every + 1) x n
		uint32_t* tape = nullptr;                    // every x n x tape_nb
		int* tape_cnt = nullptr;                     // every x n
		float2 *lam_p = nullptr, *lam_v = nullptr, *lo_p = nullptr, *lo_v = nullptr;
		float4* adj_nb = nullptr;                    // n: neighbour terms of the step being reversed
		float* dparams = nullptr;
		double* loss = nullptr;
		uint32_t* obs_list = nullptr;                // per k_adjoint warp: obs_cap entries
		int obs_cap = 0;
	} df_;
	bool diff_restore_start();
	bool diff_alloc_tape();
	bool diff_check_status();
	void diff_free();

	// trajectory output state
	std::vector<TrajWriter*> recs_;      // one per scenario (a batch writes each into its own folder)
	std::vector<int> rec_off_;           // scenario offsets of the ring's agents
	int rec_R_ = 0, rec_head_ = 0, rec_snap_head_ = 0, rec_cap_n_ = 0, rec_next_ = 0;
	float2* rec_ring_ = nullptr;
	std::vector<std::vector<double>> rec_times_;   // per scenario, each recorded step's time
	std::vector<int> rec_ids_;
	float* rec_host_[2] = { nullptr, nullptr };
	size_t rec_host_cap_[2] = { 0, 0 };
	std::atomic<int> rec_busy_[2];
	cudaEvent_t rec_ev_[2] = { nullptr, nullptr };
	bool rec_flush_async();         // after a committed sync: hand the ring to the writer
	bool rec_before_change();       // sync and flush before the agent list changes
	void rec_free();
};

}  // namespace umans
