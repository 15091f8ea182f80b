// Host tables of the cost-function plugins (plugins.hpp).
#include "plugins.hpp"

namespace umans {

// ExampleRVO: the reference's RVO cost (RVO.cpp:28-44, parameter "w",
// RVO.h:53) written as a plugin; a policy naming it behaves exactly as one
// naming "RVO".
static const PluginParam kExampleRvoParams[] = { { "w", 0, 1.0f } };

const PluginInfo kPlugins[] = {
	{ "ExampleRVO", kExampleRvoParams, 1 },
};
const int kNumPlugins = (int)(sizeof(kPlugins) / sizeof(kPlugins[0]));

}  // namespace umans
