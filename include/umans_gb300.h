/* umans_gb300: GB300 engine for the UMANS per-step agent update.
 *
 * C ABI.  Plain pointers and sizes; no CUDA or torch types.
 *
 * Part 1 is the reference's own library interface, same names, argument
 * meaning and error behaviour (src/Library/APIFunctions.h:30-113 of UMANS).
 * The reference declares its out-parameters as C++ references (float&,
 * AgentData*&, int&); at the ABI level those are pointers, as declared here,
 * so a program built against the reference header links against this
 * library unchanged.
 *
 * Part 2 is a re-entrant handle interface: any number of simulations, one
 * CUDA stream each, integer status codes (0 = success) and a per-handle
 * error string.
 */
#ifndef UMANS_GB300_H
#define UMANS_GB300_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Agent status exchanged with external applications
 * (src/Library/APIFunctions.h:33-49). */
struct AgentData {
	int id;
	float position_x;
	float position_y;
	float velocity_x;
	float velocity_y;
	float viewingDirection_x;
	float viewingDirection_y;
};

/* ---- Part 1: reference-compatible global simulation ---------------------
 * One process-wide simulation, like the reference (APIFunctions.cpp:35-45);
 * callers serialise.  nrThreads is accepted and ignored (the step runs on
 * the GPU). */

/* replaces StartSimulation, APIFunctions.h:52 / .cpp:47-70 */
bool StartSimulation(const char* configFileName, int nrThreads);
/* replaces GetSimulationTimeStep, APIFunctions.h:57 / .cpp:72-79 */
bool GetSimulationTimeStep(float* result_dt);
/* replaces DoSimulationSteps, APIFunctions.h:63 / .cpp:81-88 */
bool DoSimulationSteps(int nrSteps);
/* replaces GetAgentPositions, APIFunctions.h:71 / .cpp:90-115; the buffer is
 * owned by the library and stays valid until the next call that resizes it
 * or CleanUp. */
bool GetAgentPositions(struct AgentData** result_agentData, int* result_nrAgents);
/* replaces SetAgentPositions, APIFunctions.h:77 / .cpp:117-137 */
bool SetAgentPositions(struct AgentData* agentData, int nrAgents);
/* replaces AddAgent, APIFunctions.h:92 / .cpp:139-171 (desiredID -1 = any) */
bool AddAgent(float x, float y, float radius, float prefSpeed, float maxSpeed, float maxAcceleration,
              int policyID, int* result_id, int desiredID);
/* replaces RemoveAgent, APIFunctions.h:98 / .cpp:173-180 */
bool RemoveAgent(int id);
/* replaces SetAgentGoal, APIFunctions.h:106 / .cpp:182-194 */
bool SetAgentGoal(int id, float x, float y);
/* replaces CleanUp, APIFunctions.h:111 / .cpp:196-206 */
bool CleanUp(void);

/* ---- Part 2: handle interface --------------------------------------------
 * Each entry point replaces the reference path named beside it. */
typedef struct umans_sim umans_sim;

enum umans_status {
	UMANS_OK = 0,
	UMANS_ERR_ARGUMENT = 1,   /* null handle/pointer, bad size */
	UMANS_ERR_LOAD = 2,       /* scenario rejected (CrowdSimulator::FromConfigFile returned null) */
	UMANS_ERR_CUDA = 3,       /* CUDA runtime error */
	UMANS_ERR_DEVICE = 4,     /* device-reported condition, e.g. neighbour capacity exceeded */
	UMANS_ERR_NOT_FOUND = 5   /* unknown agent or policy id */
};

/* CrowdSimulator::FromConfigFile (crowdSimulator.cpp:516-647) */
int umans_create(const char* config_file, umans_sim** out);
/* Loads a scenario file on the host only (no device work): its agent count
 * (timed insertions included), policies and obstacle edges; the loader's
 * errors (CrowdSimulator::FromConfigFile, crowdSimulator.cpp:516-647) through
 * umans_last_error(NULL). */
int umans_scenario_info(const char* config_file, int* agents, int* policies, int* edges);
/* The loader's warnings for a scenario file (host only), one per line: the
 * messages the reference writes to standard error while loading (an invalid
 * sampling attribute, an unknown cost function, an agent without a goal, an
 * unknown world type; crowdSimulator.cpp:344-400, 516-647).  Writes up to
 * cap-1 bytes and a terminating NUL into text (may be NULL when cap is 0);
 * *needed receives the full length plus one. */
int umans_scenario_warnings(const char* config_file, char* text, int cap, int* needed);
/* The cost-function names a policy's <costfunction name="..."/> may use: the
 * built-in costs, then the compiled-in plugins (the names registered with
 * CostFunctionFactory, costFunctionFactory.cpp:41-61).  Writes up to cap
 * pointers to static strings into names (may be NULL when cap is 0) and the
 * total count into *n. */
int umans_cost_functions(const char** names, int cap, int* n);
/* as umans_create; max_neighbours <= 0 and cells_per_range <= 0 pick defaults */
int umans_create_ex(const char* config_file, int max_neighbours, float cells_per_range, int use_graph,
                    umans_sim** out);
int umans_destroy(umans_sim* sim);

/* Batched form (no counterpart in the reference, which runs one scenario per
 * process): n independent scenarios stepped together, their agents
 * concatenated in list order, scenario k at slots [offsets[k], offsets[k+1]).
 * Each scenario is simulated exactly as by umans_create on its own file.
 * Agents with a start time join the end of their scenario's agents when its
 * clock reaches it, and agents removed at their goal leave their scenario
 * (each scenario as its own simulation would), so the offsets move. */
int umans_batch_create(const char* const* config_files, int n, umans_sim** out);
/* offsets[0..nscenarios] (cap >= nscenarios + 1), either pointer may be null */
int umans_batch_offsets(umans_sim* sim, int* offsets, int cap, int* nscenarios);
/* Times the step's launch-shape candidates (cell size per interaction range,
 * warps per block, occupancy, agent-to-warp schedule, and lanes per agent,
 * 8 or 32, for force-only scenarios without obstacle edges) for trial_steps
 * each from the current state, which is restored, and keeps the fastest;
 * reports the choice (any pointer may be null). */
int umans_autotune(umans_sim* sim, int trial_steps, float* cells_per_range, int* warps_per_block,
                   float* occupancy, int* schedule, int* agent_lanes);
/* Applies a launch shape, such as one umans_autotune chose: cells per
 * interaction range (> 0), warps per block (1..8), occupancy (0, 1],
 * schedule (0 interleaved, 1 contiguous, 2 work list), lanes per agent (8 or
 * 32).  Results do not depend on it.  UMANS_ERR_ARGUMENT when out of range. */
int umans_set_launch(umans_sim* sim, float cells_per_range, int warps_per_block, float occupancy, int schedule,
                     int agent_lanes);
/* Small worlds (one scenario, at most 4096 agents, neighbour lists that fit
 * in shared memory) whose policies run the general, ORCA or
 * Karamouzas-sampling kernel: with enable != 0 (the default) the steps of
 * one umans_step / umans_step_async call run in one cooperative launch (one
 * block builds each step's grid, then every block updates its agents); with
 * 0, one graph launch per step.  Steps that need host work in between
 * (trajectory output, agents joining or leaving) take one launch each
 * either way.  Results do not depend on it. */
int umans_set_multi_step(umans_sim* sim, int enable);
/* CrowdSimulator::RunSimulationSteps (crowdSimulator.cpp:77-95): n steps,
 * waits for them, reports device-side errors */
int umans_step(umans_sim* sim, int nsteps);
/* enqueue n steps on the simulation's stream without waiting */
int umans_step_async(umans_sim* sim, int nsteps);
int umans_synchronize(umans_sim* sim);
int umans_num_agents(umans_sim* sim, int* n);
int umans_time(umans_sim* sim, double* t);          /* WorldBase::GetCurrentTime */
int umans_dt(umans_sim* sim, float* dt);            /* WorldBase::GetDeltaTime */
int umans_end_time(umans_sim* sim, float* t);       /* scenario end_time (FLT_MAX if absent) */
/* state in list order (WorldBase::GetAgents): ids[n], pos/vel/viewdir[2n];
 * any pointer may be null; cap = capacity in agents */
int umans_get_state(umans_sim* sim, int* ids, float* pos, float* vel, float* viewdir, int cap);
/* preferred velocities and goals of the last step, [2n] each (may be null) */
int umans_get_aux(umans_sim* sim, float* prefvel, float* goal, int cap);
/* overwrite pos/vel/viewdir of all agents, list order (Agent::setPosition,
 * Agent::setVelocity_ExternalApplication); null pointers leave a field */
int umans_set_state(umans_sim* sim, const float* pos, const float* vel, const float* viewdir);
/* SetAgentPositions (APIFunctions.cpp:117-137): by id, unknown ids skipped */
int umans_set_agents(umans_sim* sim, const struct AgentData* agents, int n);
/* GetAgentPositions (APIFunctions.cpp:90-115) into a caller buffer of cap records */
int umans_get_agents(umans_sim* sim, struct AgentData* out, int cap, int* n);
int umans_add_agent(umans_sim* sim, float x, float y, float radius, float pref_speed, float max_speed,
                    float max_acceleration, int policy_id, int desired_id, int* out_id);
int umans_remove_agent(umans_sim* sim, int id);
int umans_set_goal(umans_sim* sim, int id, float x, float y);
/* Neighbour lists the next step uses (Agent::ComputeNeighbors,
 * agent.cpp:43-50): per agent in list order, up to `cap` neighbour ids and
 * PhantomAgent distSqr values at [i*cap, i*cap+cap); counts[i] = full length. */
int umans_neighbours(umans_sim* sim, int cap, int* ids, float* dist2, int* counts);
/* neighbour-list capacity in use (entries per agent) */
int umans_max_neighbours(umans_sim* sim, int* cap);
/* the CUDA stream (cudaStream_t) the steps run on, for event timing */
int umans_stream(umans_sim* sim, void** stream);
/* device addresses of the float2 position / velocity arrays (list order) */
int umans_device_state(umans_sim* sim, void** pos, void** vel);
/* Profiling: when enabled, each step runs without the CUDA graph and is
 * bracketed by CUDA events on the simulation's stream (whole step, the grid
 * build k_bbox..k_scatter, and the fused per-agent kernels); totals
 * accumulate until the next umans_profile. */
int umans_profile(umans_sim* sim, int enable);
int umans_profile_totals(umans_sim* sim, double* agent_kernel_ms, double* step_ms, int* steps,
                         int* kernels_per_step, double* grid_build_ms);
/* Work counters of the profiled steps (since umans_profile(sim, 1)), first n
 * of: Karamouzas samples inside the deviation/speed window (the samples whose
 * collision times are swept, Karamouzas.cpp:39-44), pair collision times
 * evaluated for them, agents through that sampling path. */
int umans_profile_counters(umans_sim* sim, unsigned long long* counts, int n);
/* Differentiable form (no counterpart in the reference), for calibrating
 * force-model parameters against observed trajectories.  Supported policies:
 * method "gradient" with SocialForcesAvoidance, PowerLaw and
 * GoalReachingForce costs (ForceBasedFunction::GetGradient,
 * src/Engine/CostFunctions/ForceBasedFunction.cpp:32-36), contact forces
 * and static obstacles (SocialForcesAvoidance.cpp:112-140, policy.cpp:126-137)
 * included; a fixed agent set.
 *
 * umans_diff_begin records the current state as the episode's start and the
 * targets (steps x n x 2 floats, list order); the loss of an episode is
 *   L = weight * sum_{t=1..steps} sum_i |p_i(t) - target_i(t)|^2
 * (weight <= 0: 1 / (steps * n)).  umans_diff_forward runs the episode from
 * its start, keeping a checkpoint every checkpoint_every steps, and returns
 * L.  umans_diff_backward recomputes each segment from its checkpoint with
 * the neighbour lists recorded, reverses it (hand-written adjoint), writes
 * dL/d(V0, sigma, k, tau0) per scenario into dparams[4 * nscenarios] and,
 * where non-null, dL/d(initial positions) and dL/d(initial velocities)
 * (n x 2 floats each), and puts the simulation back in the start state.
 * Neighbour lists and branches (cut-offs, clamps, the view-angle factor) are
 * those of the forward pass: the gradient is that of the piecewise-smooth
 * step map on the piece the episode lies in. */
int umans_diff_begin(umans_sim* sim, int steps, int checkpoint_every, const float* targets, float weight);
int umans_diff_forward(umans_sim* sim, double* loss);
int umans_diff_backward(umans_sim* sim, float* dparams, float* dpos0, float* dvel0);
int umans_diff_end(umans_sim* sim);
/* (V0, sigma) of every SocialForcesAvoidance cost and (k, tau0) of every
 * PowerLaw cost of scenario `scenario` (all scenarios when < 0); NaN entries
 * are left unchanged.  get: NaN where the scenario has no such cost. */
int umans_set_force_params(umans_sim* sim, int scenario, const float* params4);
int umans_get_force_params(umans_sim* sim, int scenario, float* params4);
/* Trajectory output, the reference's CSVWriter (src/Engine/tools/csvwriter.cpp,
 * fed after every step by CrowdSimulator::RunSimulationSteps,
 * crowdSimulator.cpp:77-95).  After every step the positions go to a device
 * ring of ring_steps steps; a full ring is copied to page-locked host memory
 * and written by a background thread while the GPU keeps stepping.  binary = 0:
 * the reference's layout, one file output_<id>.csv per agent with "t,x,y"
 * lines appended, at full float precision (9 significant digits; the
 * reference writes 6); binary = 1: one file trajectory.bin of chunks (see
 * umans_gb300.read_trajectory).  Changes of the agent list flush the ring
 * first.  A batch writes scenario k into directory/scenario_k, as a
 * simulation of that scenario alone would.  umans_record_flush writes everything
 * recorded so far and waits; umans_record_stop flushes and ends recording
 * (also done by umans_destroy). */
int umans_record_start(umans_sim* sim, const char* directory, int ring_steps, int binary);
int umans_record_flush(umans_sim* sim);
int umans_record_stop(umans_sim* sim);
/* Test hook: the device's exponential used by the force models, which
 * returns exactly the host C library's expf for x in [-87, 0]; evaluates n
 * values and reports the size of the exception table.  Errors are reported
 * through umans_last_error(NULL). */
int umans_debug_ref_expf(const float* x, float* y, int n, size_t* exceptions);
/* Test hook: checks the short exponential that the force models try first
 * against the table-backed one, over the float bit patterns
 * [first, first + count) that lie in [-87, 0]: counts[0] = values it
 * answered, counts[1] = answered values whose result differs (must be 0),
 * counts[2] = answered values listed in the exception table (must be 0);
 * *band (may be null) receives the table's midpoint band in ulps.  Errors
 * are reported through umans_last_error(NULL). */
int umans_debug_expf_check(unsigned int first, unsigned int count, unsigned long long* counts, float* band);
/* Test hook: the device's sinf/cosf, which return exactly the host C
 * library's sinf/cosf for |x| <= 64 (the float sin/cos of
 * costFunction.cpp:33, :104, :321 and FOEAvoidance.cpp:142); evaluates n
 * values and reports the size of the exception tables.  Errors:
 * umans_last_error(NULL). */
int umans_debug_ref_sincosf(const float* x, float* s, float* c, int n, size_t* exceptions);
/* Test hook: the device's (float)((double)a*b - (double)c*d) on n quadruples
 * abcd[4*i .. 4*i+3] (the promoted products of SocialForcesAvoidance.cpp:86
 * and vector2D.h:166-170).  Errors: umans_last_error(NULL). */
int umans_debug_prod_diff(const float* abcd, float* y, int n);
/* ORCA velocities without allocation.  No counterpart in the reference.
 *
 * For callers that cannot allocate GPU memory at the moment they need a
 * result, for instance an application that hands all device memory out
 * through its own pool at start-up and forbids cudaMalloc afterwards, or code
 * running while another component owns the device allocator.  Computes, for n
 * agents of an infinite world whose data the caller keeps on the device, the
 * new velocity of the ORCA policy with the global method
 * (Policy::ComputeNewVelocity with ORCA::GetGlobalMinimum), writing new_vel.
 * It calls no cudaMalloc/cudaFree and no allocating routine: the ORCA line
 * buffers are a file-scope device array of 1 MiB.
 *
 * Device pointers: pos, vel, pref, new_vel are float2[n]; radius, max_speed,
 * max_accel are float[n]; nbr_index / nbr_dist2 are [n * nbr_cap] (neighbour
 * list index into the same arrays, and PhantomAgent distSqr), nbr_count[n].
 * Limit: nbr_cap <= 128 (lines per agent); larger is rejected with
 * UMANS_ERR_ARGUMENT.  A count above nbr_cap (the list is truncated) or a
 * neighbour index outside [0, n) (the entry is skipped) returns
 * UMANS_ERR_DEVICE.  The first call on a device looks up the array's device
 * address.  Every call reads a status word back and synchronises `stream`
 * (a cudaStream_t, may be null), so it must not be called while that stream
 * is being captured.  All calls share the array: calls that overlap on the
 * GPU race and must be serialised.  Errors: umans_last_error(NULL), per
 * host thread. */
int umans_orca_velocities_noalloc(int n, const float* pos, const float* vel, const float* pref,
                                  const float* radius, const float* max_speed, const float* max_accel,
                                  const int* nbr_index, const float* nbr_dist2, const int* nbr_count,
                                  int nbr_cap, float range, float time_horizon, float dt,
                                  float relaxation_time, float* new_vel, void* stream);
/* the last error of this handle, or of the last failed umans_create when sim is null */
const char* umans_last_error(umans_sim* sim);

#ifdef __cplusplus
}
#endif
#endif
