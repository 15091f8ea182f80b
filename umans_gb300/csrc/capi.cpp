// C ABI of the engine (include/umans_gb300.h).
#include "../../include/umans_gb300.h"

#include <cfloat>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.hpp"

using umans::Engine;

struct umans_sim {
	Engine* eng = nullptr;
	std::string err;
};

static thread_local std::string g_create_error;
static thread_local bool g_last_error_noalloc = false;

namespace umans {
int orca_velocities_noalloc(int n, const float* pos, const float* vel, const float* pref, const float* radius,
                            const float* max_speed, const float* max_accel, const int* nbr_index,
                            const float* nbr_dist2, const int* nbr_count, int nbr_cap, float range,
                            float time_horizon, float dt, float relaxation_time, float* new_vel, void* stream);
const char* noalloc_last_error();
}

static int fail(umans_sim* s, int code, const std::string& msg)
{
	if (s) s->err = msg;
	else { g_create_error = msg; g_last_error_noalloc = false; }
	return code;
}

extern "C" {

int umans_create_ex(const char* config_file, int max_neighbours, float cells_per_range, int use_graph, umans_sim** out)
{
	if (!config_file || !out) return fail(nullptr, UMANS_ERR_ARGUMENT, "null argument");
	*out = nullptr;
	umans::EngineOptions opt;
	if (max_neighbours > 0) opt.max_neighbours = max_neighbours;
	if (cells_per_range > 0) opt.cells_per_range = cells_per_range;
	opt.use_graph = use_graph != 0;
	std::string err;
	Engine* e = Engine::create(config_file, err, opt);
	if (!e) return fail(nullptr, UMANS_ERR_LOAD, err);
	umans_sim* s = new umans_sim();
	s->eng = e;
	*out = s;
	return UMANS_OK;
}

int umans_scenario_info(const char* config_file, int* agents, int* policies, int* edges)
{
	if (!config_file) return fail(nullptr, UMANS_ERR_ARGUMENT, "null argument");
	umans::Scenario sc;
	std::string err;
	if (!umans::load_scenario(config_file, sc, err)) return fail(nullptr, UMANS_ERR_LOAD, err);
	if (agents) *agents = (int)sc.agents.size();
	if (policies) *policies = (int)sc.policies.size();
	if (edges) *edges = (int)sc.edges.size();
	return UMANS_OK;
}

int umans_scenario_warnings(const char* config_file, char* text, int cap, int* needed)
{
	if (!config_file || !needed || cap < 0 || (cap > 0 && !text))
		return fail(nullptr, UMANS_ERR_ARGUMENT, "bad argument");
	umans::Scenario sc;
	std::string err;
	if (!umans::load_scenario(config_file, sc, err)) return fail(nullptr, UMANS_ERR_LOAD, err);
	std::string all;
	for (const auto& w : sc.warnings) all += w + "\n";
	*needed = (int)all.size() + 1;
	if (cap > 0) {
		const size_t k = std::min(all.size(), (size_t)cap - 1);
		std::memcpy(text, all.data(), k);
		text[k] = 0;
	}
	return UMANS_OK;
}

int umans_cost_functions(const char** names, int cap, int* n)
{
	if (!n || cap < 0 || (cap > 0 && !names)) return fail(nullptr, UMANS_ERR_ARGUMENT, "bad argument");
	const int total = umans::cost_function_count();
	for (int k = 0; k < total && k < cap; ++k) names[k] = umans::cost_function_name(k);
	*n = total;
	return UMANS_OK;
}

int umans_batch_create(const char* const* config_files, int n, umans_sim** out)
{
	if (!config_files || n <= 0 || !out) return fail(nullptr, UMANS_ERR_ARGUMENT, "bad argument");
	*out = nullptr;
	std::vector<std::string> files;
	for (int k = 0; k < n; ++k) {
		if (!config_files[k]) return fail(nullptr, UMANS_ERR_ARGUMENT, "null file name");
		files.emplace_back(config_files[k]);
	}
	std::string err;
	Engine* e = Engine::create_batch(files, err);
	if (!e) return fail(nullptr, UMANS_ERR_LOAD, err);
	umans_sim* s = new umans_sim();
	s->eng = e;
	*out = s;
	return UMANS_OK;
}

int umans_batch_offsets(umans_sim* s, int* offsets, int cap, int* nscenarios)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	const int ns = s->eng->num_scenarios();
	if (nscenarios) *nscenarios = ns;
	if (offsets) {
		if (cap < ns + 1) return fail(s, UMANS_ERR_ARGUMENT, "offsets buffer needs nscenarios + 1 entries");
		for (int k = 0; k <= ns; ++k) offsets[k] = s->eng->scenario_offset(k);
	}
	return UMANS_OK;
}

int umans_set_launch(umans_sim* s, float cells_per_range, int warps_per_block, float occupancy, int schedule,
                     int agent_lanes)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	umans::EngineOptions o;
	o.cells_per_range = cells_per_range;
	o.warps_per_block = warps_per_block;
	o.occupancy = occupancy;
	o.schedule = schedule;
	o.agent_lanes = agent_lanes;
	if (!s->eng->set_launch(o)) return fail(s, UMANS_ERR_ARGUMENT, s->eng->error());
	return UMANS_OK;
}

int umans_set_multi_step(umans_sim* s, int enable)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->set_multi_step(enable != 0)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	return UMANS_OK;
}

int umans_autotune(umans_sim* s, int trial_steps, float* cells_per_range, int* warps_per_block, float* occupancy,
                   int* schedule, int* agent_lanes)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	umans::EngineOptions o;
	if (!s->eng->autotune(trial_steps, &o)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	if (cells_per_range) *cells_per_range = o.cells_per_range;
	if (warps_per_block) *warps_per_block = o.warps_per_block;
	if (occupancy) *occupancy = o.occupancy;
	if (schedule) *schedule = o.schedule;
	if (agent_lanes) *agent_lanes = o.agent_lanes;
	return UMANS_OK;
}

int umans_create(const char* config_file, umans_sim** out)
{
	return umans_create_ex(config_file, 0, 0, 1, out);
}

int umans_destroy(umans_sim* s)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	delete s->eng;
	delete s;
	return UMANS_OK;
}

int umans_step_async(umans_sim* s, int n)
{
	if (!s || n < 0) return fail(s, UMANS_ERR_ARGUMENT, "bad argument");
	if (!s->eng->step(n)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	return UMANS_OK;
}

int umans_synchronize(umans_sim* s)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->sync()) return fail(s, UMANS_ERR_DEVICE, s->eng->error());
	return UMANS_OK;
}

int umans_step(umans_sim* s, int n)
{
	int rc = umans_step_async(s, n);
	if (rc) return rc;
	return umans_synchronize(s);
}

int umans_num_agents(umans_sim* s, int* n)
{
	if (!s || !n) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	*n = s->eng->num_agents();
	return UMANS_OK;
}

int umans_time(umans_sim* s, double* t)
{
	if (!s || !t) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	*t = s->eng->time();
	return UMANS_OK;
}

int umans_dt(umans_sim* s, float* dt)
{
	if (!s || !dt) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	*dt = s->eng->dt();
	return UMANS_OK;
}

int umans_end_time(umans_sim* s, float* t)
{
	if (!s || !t) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	*t = s->eng->end_time();
	return UMANS_OK;
}

int umans_get_state(umans_sim* s, int* ids, float* pos, float* vel, float* viewdir, int cap)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (cap < s->eng->num_agents()) return fail(s, UMANS_ERR_ARGUMENT, "buffer smaller than the number of agents");
	if (!s->eng->get_state(ids, pos, vel, viewdir)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	return UMANS_OK;
}

int umans_get_aux(umans_sim* s, float* prefvel, float* goal, int cap)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (cap < s->eng->num_agents()) return fail(s, UMANS_ERR_ARGUMENT, "buffer smaller than the number of agents");
	if (!s->eng->get_state(nullptr, nullptr, nullptr, nullptr, prefvel, goal)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	return UMANS_OK;
}

int umans_set_state(umans_sim* s, const float* pos, const float* vel, const float* viewdir)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->set_state(pos, vel, viewdir)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	return UMANS_OK;
}

int umans_set_agents(umans_sim* s, const AgentData* a, int n)
{
	if (!s || (n > 0 && !a)) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	static_assert(sizeof(AgentData) == sizeof(umans::AgentRecord), "AgentData layout");
	if (!s->eng->set_agent_data(a, n)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	return UMANS_OK;
}

int umans_get_agents(umans_sim* s, AgentData* out, int cap, int* n)
{
	if (!s || !out || !n) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	if (cap < s->eng->num_agents()) return fail(s, UMANS_ERR_ARGUMENT, "buffer smaller than the number of agents");
	if (!s->eng->get_agent_data(out)) return fail(s, UMANS_ERR_CUDA, s->eng->error());
	*n = s->eng->num_agents();
	return UMANS_OK;
}

int umans_add_agent(umans_sim* s, float x, float y, float radius, float pref_speed, float max_speed,
                    float max_acceleration, int policy_id, int desired_id, int* out_id)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->add_agent(x, y, radius, pref_speed, max_speed, max_acceleration, policy_id, desired_id, out_id))
		return fail(s, UMANS_ERR_NOT_FOUND, s->eng->error());
	return UMANS_OK;
}

int umans_remove_agent(umans_sim* s, int id)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->remove_agent(id)) return fail(s, UMANS_ERR_NOT_FOUND, s->eng->error());
	return UMANS_OK;
}

int umans_set_goal(umans_sim* s, int id, float x, float y)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->set_goal(id, x, y)) return fail(s, UMANS_ERR_NOT_FOUND, s->eng->error());
	return UMANS_OK;
}

int umans_neighbours(umans_sim* s, int cap, int* ids, float* dist2, int* counts)
{
	if (!s || cap < 0) return fail(s, UMANS_ERR_ARGUMENT, "bad argument");
	if (!s->eng->neighbours(cap, ids, dist2, counts)) return fail(s, UMANS_ERR_DEVICE, s->eng->error());
	return UMANS_OK;
}

int umans_max_neighbours(umans_sim* s, int* cap)
{
	if (!s || !cap) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	*cap = s->eng->max_neighbours();
	return UMANS_OK;
}

int umans_stream(umans_sim* s, void** stream)
{
	if (!s || !stream) return fail(s, UMANS_ERR_ARGUMENT, "null argument");
	*stream = (void*)s->eng->stream();
	return UMANS_OK;
}

int umans_device_state(umans_sim* s, void** pos, void** vel)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (pos) *pos = s->eng->device_positions();
	if (vel) *vel = s->eng->device_velocities();
	return UMANS_OK;
}

int umans_profile(umans_sim* s, int enable)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	s->eng->set_profile(enable != 0);
	return UMANS_OK;
}

int umans_profile_counters(umans_sim* s, unsigned long long* counts, int n)
{
	if (!s || (n > 0 && !counts)) return UMANS_ERR_ARGUMENT;
	if (!s->eng->profile_counters(counts, n)) return fail(s, UMANS_ERR_DEVICE, s->eng->error());
	return UMANS_OK;
}

int umans_profile_totals(umans_sim* s, double* agent_kernel_ms, double* step_ms, int* steps, int* kernels_per_step,
                         double* grid_build_ms)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	double a = 0, b = 0, g = 0;
	int n = 0;
	s->eng->profile_totals(&a, &b, &n, &g);
	if (grid_build_ms) *grid_build_ms = g;
	if (agent_kernel_ms) *agent_kernel_ms = a;
	if (step_ms) *step_ms = b;
	if (steps) *steps = n;
	if (kernels_per_step) *kernels_per_step = s->eng->kernels_per_step();
	return UMANS_OK;
}

int umans_diff_begin(umans_sim* s, int steps, int checkpoint_every, const float* targets, float weight)
{
	if (!s || steps <= 0 || checkpoint_every <= 0 || (!targets && s->eng->num_agents() > 0))
		return UMANS_ERR_ARGUMENT;
	if (!s->eng->diff_begin(steps, checkpoint_every, targets, weight))
		return fail(s, UMANS_ERR_ARGUMENT, s->eng->error());
	return UMANS_OK;
}

int umans_diff_forward(umans_sim* s, double* loss)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->diff_forward(loss)) return fail(s, UMANS_ERR_DEVICE, s->eng->error());
	return UMANS_OK;
}

int umans_diff_backward(umans_sim* s, float* dparams, float* dpos0, float* dvel0)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->diff_backward(dparams, dpos0, dvel0)) return fail(s, UMANS_ERR_DEVICE, s->eng->error());
	return UMANS_OK;
}

int umans_diff_end(umans_sim* s)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	s->eng->diff_end();
	return UMANS_OK;
}

int umans_set_force_params(umans_sim* s, int scenario, const float* params4)
{
	if (!s || !params4) return UMANS_ERR_ARGUMENT;
	if (!s->eng->set_force_params(scenario, params4)) return fail(s, UMANS_ERR_ARGUMENT, s->eng->error());
	return UMANS_OK;
}

int umans_get_force_params(umans_sim* s, int scenario, float* params4)
{
	if (!s || !params4) return UMANS_ERR_ARGUMENT;
	if (!s->eng->get_force_params(scenario, params4)) return fail(s, UMANS_ERR_ARGUMENT, s->eng->error());
	return UMANS_OK;
}

int umans_record_start(umans_sim* s, const char* directory, int ring_steps, int binary)
{
	if (!s || !directory) return UMANS_ERR_ARGUMENT;
	if (!s->eng->record_start(directory, ring_steps, binary ? umans::TrajWriter::BINARY : umans::TrajWriter::CSV))
		return fail(s, UMANS_ERR_ARGUMENT, s->eng->error());
	return UMANS_OK;
}

int umans_record_flush(umans_sim* s)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->record_flush()) return fail(s, UMANS_ERR_DEVICE, s->eng->error());
	return UMANS_OK;
}

int umans_record_stop(umans_sim* s)
{
	if (!s) return UMANS_ERR_ARGUMENT;
	if (!s->eng->record_stop()) return fail(s, UMANS_ERR_DEVICE, s->eng->error());
	return UMANS_OK;
}

int umans_debug_ref_expf(const float* x, float* y, int n, size_t* exceptions)
{
	if ((n > 0 && (!x || !y)) || n < 0) return fail(nullptr, UMANS_ERR_ARGUMENT, "bad argument");
	std::string err;
	if (!umans::debug_ref_expf(x, y, n, exceptions, err)) return fail(nullptr, UMANS_ERR_CUDA, err);
	return UMANS_OK;
}

int umans_debug_expf_check(unsigned int first, unsigned int count, unsigned long long* counts, float* band)
{
	if (!counts) return fail(nullptr, UMANS_ERR_ARGUMENT, "bad argument");
	std::string err;
	if (!umans::debug_expf_check(first, count, counts, band, err)) return fail(nullptr, UMANS_ERR_CUDA, err);
	return UMANS_OK;
}

int umans_debug_ref_sincosf(const float* x, float* s, float* c, int n, size_t* exceptions)
{
	if ((n > 0 && (!x || !s || !c)) || n < 0) return fail(nullptr, UMANS_ERR_ARGUMENT, "bad argument");
	std::string err;
	if (!umans::debug_ref_sincosf(x, s, c, n, exceptions, err)) return fail(nullptr, UMANS_ERR_CUDA, err);
	return UMANS_OK;
}

int umans_debug_prod_diff(const float* abcd, float* y, int n)
{
	if ((n > 0 && (!abcd || !y)) || n < 0) return fail(nullptr, UMANS_ERR_ARGUMENT, "bad argument");
	std::string err;
	if (!umans::debug_prod_diff(abcd, y, n, err)) return fail(nullptr, UMANS_ERR_CUDA, err);
	return UMANS_OK;
}

int umans_orca_velocities_noalloc(int n, const float* pos, const float* vel, const float* pref, const float* radius,
                                  const float* max_speed, const float* max_accel, const int* nbr_index,
                                  const float* nbr_dist2, const int* nbr_count, int nbr_cap, float range,
                                  float time_horizon, float dt, float relaxation_time, float* new_vel, void* stream)
{
	// no std::string here: this path must not allocate
	const int rc = umans::orca_velocities_noalloc(n, pos, vel, pref, radius, max_speed, max_accel, nbr_index,
	                                              nbr_dist2, nbr_count, nbr_cap, range, time_horizon, dt,
	                                              relaxation_time, new_vel, stream);
	if (rc != 0) g_last_error_noalloc = true;
	return rc;
}

const char* umans_last_error(umans_sim* s)
{
	if (s) return s->err.c_str();
	return g_last_error_noalloc ? umans::noalloc_last_error() : g_create_error.c_str();
}

// ---------------------------------------------------------------------------
// reference-compatible global interface (src/Library/APIFunctions.cpp)
// ---------------------------------------------------------------------------
static umans_sim* g_sim = nullptr;
// the AgentData buffer GetAgentPositions hands out (library-owned, valid
// until the next resize or CleanUp), page-locked so that the device writes
// it directly
struct AgentBuffer {
	AgentData* p = nullptr;
	size_t cap = 0;
	size_t size() const { return cap; }
	AgentData* data() { return p; }
	void release()
	{
		if (p) cudaFreeHost(p);
		p = nullptr;
		cap = 0;
	}
};
static AgentBuffer g_agent_data;

// resizeAgentData: APIFunctions.cpp:37-45 (power-of-two capacity)
static bool resize_agent_data(size_t n)
{
	size_t cap = (size_t)std::pow(2, 1 + (int)std::ceil(std::log2((double)std::max<size_t>(n, 1))));
	g_agent_data.release();
	if (cudaMallocHost(&g_agent_data.p, sizeof(AgentData) * cap) != cudaSuccess) {
		g_agent_data.p = nullptr;
		return false;
	}
	std::memset(g_agent_data.p, 0, sizeof(AgentData) * cap);
	g_agent_data.cap = cap;
	return true;
}

bool StartSimulation(const char* configFileName, int nrThreads)
{
	(void)nrThreads;
	if (g_sim) { umans_destroy(g_sim); g_sim = nullptr; }
	if (umans_create(configFileName, &g_sim) != UMANS_OK) {
		g_sim = nullptr;
		return false;
	}
	resize_agent_data(g_sim->eng->num_agents());
	return true;
}

bool GetSimulationTimeStep(float* result_dt)
{
	if (!g_sim || !result_dt) return false;
	*result_dt = g_sim->eng->dt();
	return true;
}

bool DoSimulationSteps(int nrSteps)
{
	if (!g_sim) return false;
	return umans_step(g_sim, nrSteps) == UMANS_OK;
}

bool GetAgentPositions(AgentData** result_agentData, int* result_nrAgents)
{
	if (!g_sim || !result_agentData || !result_nrAgents) return false;
	const size_t n = (size_t)g_sim->eng->num_agents();
	if ((n > g_agent_data.size() || n * 4 < g_agent_data.size()) && !resize_agent_data(n)) return false;
	if (!g_sim->eng->get_agent_data(g_agent_data.data())) return false;
	*result_agentData = g_agent_data.data();
	*result_nrAgents = (int)n;
	return true;
}

bool SetAgentPositions(AgentData* agentData, int nrAgents)
{
	// the reference dereferences its simulation without a null check
	// (APIFunctions.cpp:117-137); here a missing simulation returns false
	if (!g_sim) return false;
	return umans_set_agents(g_sim, agentData, nrAgents) == UMANS_OK;
}

bool AddAgent(float x, float y, float radius, float prefSpeed, float maxSpeed, float maxAcceleration, int policyID,
              int* result_id, int desiredID)
{
	if (!g_sim) return false;
	int id = -1;
	if (umans_add_agent(g_sim, x, y, radius, prefSpeed, maxSpeed, maxAcceleration, policyID, desiredID, &id) != UMANS_OK)
		return false;
	if (result_id) *result_id = id;
	return true;
}

bool RemoveAgent(int id)
{
	if (!g_sim) return false;
	return umans_remove_agent(g_sim, id) == UMANS_OK;
}

bool SetAgentGoal(int id, float x, float y)
{
	if (!g_sim) return false;
	return umans_set_goal(g_sim, id, x, y) == UMANS_OK;
}

bool CleanUp(void)
{
	if (!g_sim) return false;
	umans_destroy(g_sim);
	g_sim = nullptr;
	g_agent_data.release();
	return true;
}

}  // extern "C"
