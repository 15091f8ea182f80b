// Scenario loading with the semantics of CrowdSimulator::FromConfigFile
// (src/Engine/core/crowdSimulator.cpp:516-647) and its helpers.
#pragma once
#include <string>
#include <vector>

#include <vector_types.h>

#include "model.hpp"

namespace umans {

struct AgentInit {
	int id;
	float x, y, gx, gy;
	float radius, pref_speed, max_speed, max_accel;
	int policy;          // index into Scenario::policies
	float start_time;
	bool remove_at_goal;
	int scen = 0;        // the scenario of a batch it belongs to (set by the engine)
};

struct Scenario {
	int world = W_INFINITE;
	float width = 0, height = 0;
	float dt = -1;
	float end_time;      // MaxFloat when absent (crowdSimulator.cpp:33)
	std::vector<PolicyDesc> policies;
	std::vector<int> policy_ids;
	std::vector<AgentInit> agents;   // in the order the reference adds them
	// obstacle edges (a.x, a.y, b.x, b.y): every polygon's closed outline,
	// polygons in file order (Polygon2D::Polygon2D, tools/Polygon2D.cpp:27-35)
	std::vector<float4> edges;
	int next_unused_id = 0;
	std::vector<std::string> warnings;
};

// Returns false and fills `error` when the reference would fail to load.
bool load_scenario(const std::string& path, Scenario& out, std::string& error);

// Fills the defaults of a cost function of the given kind (reference headers).
void cost_defaults(int kind, CostDesc& c);
// Name -> kind, or -1 for names the reference does not register, or -2 for
// names the reference registers but this engine does not run.
int cost_kind_from_name(const std::string& name);
const char* cost_kind_name(int kind);
// every registered cost-function name: built-in kinds, then plugins
int cost_function_count();
const char* cost_function_name(int index);

}  // namespace umans
