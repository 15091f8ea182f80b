// Host tables of the cost-function plugins (plugins.hpp).
#include "plugins.hpp"

#include "model.hpp"

namespace umans {

// every parameter slot indexes CostDesc::p
template <int N>
constexpr bool slots_in_range(const PluginParam (&params)[N])
{
	for (int k = 0; k < N; ++k)
		if (params[k].slot < 0 || params[k].slot >= (int)(sizeof(CostDesc::p) / sizeof(float))) return false;
	return true;
}

// ExampleRVO: the reference's RVO cost (RVO.cpp:28-44, parameter "w",
// RVO.h:53) written as a plugin; a policy naming it behaves exactly as one
// naming "RVO".
static constexpr PluginParam kExampleRvoParams[] = { { "w", 0, 1.0f } };
static_assert(slots_in_range(kExampleRvoParams), "ExampleRVO parameter slot outside CostDesc::p");

// ExampleFOE: the reference's FOEAvoidance (FOEAvoidance.cpp:50-143, no
// parameters of its own) as a plugin with its closed-form gradient.
// ExampleGoal: GoalReachingForce as the ForceBasedFunction it is
// (ForceBasedFunction.cpp:26-52, GoalReachingForce.cpp:26-29, agentMass,
// range 0 as GoalReachingForce.h:38 sets it), with its gradient and its
// closed-form global minimum.
static constexpr PluginParam kExampleGoalParams[] = { { "agentMass", 5, 1.0f } };
static_assert(slots_in_range(kExampleGoalParams), "ExampleGoal parameter slot outside CostDesc::p");

const PluginInfo kPlugins[] = {
	{ "ExampleRVO", kExampleRvoParams, 1, -1.0f, false, false },
	{ "ExampleFOE", nullptr, 0, -1.0f, true, false },
	{ "ExampleGoal", kExampleGoalParams, 1, 0.0f, true, true },
};
const int kNumPlugins = (int)(sizeof(kPlugins) / sizeof(kPlugins[0]));
static_assert(sizeof(kPlugins) / sizeof(kPlugins[0]) == kPluginCount, "kPluginCount must count kPlugins");

}  // namespace umans
