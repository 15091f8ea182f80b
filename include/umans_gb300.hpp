/* umans_gb300.hpp — C++ mirror of the reference's policy and world
 * construction over the C ABI of umans_gb300.h (header only, C++17).
 *
 * The reference builds a simulation in C++: Policy(OptimizationMethod,
 * SamplingParameters) and Policy::AddCostFunction (src/Engine/core/policy.h:
 * 100-152), a WorldInfinite or WorldToric (src/Engine/core/worldInfinite.h,
 * worldToric.h) with its agents and obstacles, stepped by CrowdSimulator.
 * This engine loads every simulation from the scenario format, so the
 * classes below compose that format: a Policy writes the <Policy> element
 * the loader (CrowdSimulator::FromConfigFile_loadSinglePolicy,
 * crowdSimulator.cpp:327-422) reads back into the same policy, a World
 * writes the whole scenario, and a Simulation owns the engine handle made
 * from it.  Attributes left unset are not written, so the loader applies the
 * reference's defaults.  Cost functions are named as registered
 * (umans_cost_functions: the built-ins, then the plugins).
 *
 *     umans::Policy p(0, umans::OptimizationMethod::GRADIENT);
 *     p.setRelaxationTime(0.5f);
 *     p.AddCostFunction("SocialForcesAvoidance", {}, 5.0f);
 *     p.AddCostFunction("GoalReachingForce");
 *     umans::World w(umans::WorldType::Toric, 0.1f, 400, 400);
 *     w.AddPolicy(p);
 *     w.AddAgent({ -10, 0 }, { 10, 0 });
 *     umans::Simulation sim(w.Write("/tmp/scenario.xml"));
 *     sim.Step(100);
 *
 * Errors (an unknown method or sampling choice, a fifth cost function, an
 * engine error) throw std::runtime_error with the engine's message.
 */
#ifndef UMANS_GB300_HPP
#define UMANS_GB300_HPP

#include <cstdio>
#include <fstream>
#include <map>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "umans_gb300.h"

namespace umans {

/* Policy::OptimizationMethod (policy.h:100-111) */
enum class OptimizationMethod { GRADIENT, SAMPLING, GLOBAL };

inline const char* to_string(OptimizationMethod m)
{
	return m == OptimizationMethod::GRADIENT ? "gradient" : m == OptimizationMethod::SAMPLING ? "sampling" : "global";
}

/* a float as the scenario writers print it: the shortest round trip of the
 * float (9 significant digits) */
inline std::string format_float(float x)
{
	char b[32];
	std::snprintf(b, sizeof(b), "%.9g", (double)x);
	return b;
}

/* SamplingParameters (policy.h:36-87); an unset field keeps the reference's
 * default (regular, base zero, base direction current velocity, radius
 * preferred speed, 180 degrees, 4 speeds x 11 angles, 100 random samples,
 * base not included) */
struct SamplingParameters {
	std::optional<std::string> type;             /* "regular" | "random" */
	std::optional<std::string> base;             /* "zero" | "current velocity" */
	std::optional<std::string> baseDirection;    /* "unit" | "current velocity" | "preferred velocity" */
	std::optional<std::string> radius;           /* "preferred speed" | "maximum speed" | "maximum acceleration" */
	std::optional<float> angle;                  /* degrees */
	std::optional<int> speedSamples, angleSamples, randomSamples;
	std::optional<bool> includeBaseAsSample;

	/* SamplingParameters::ApproximateGlobalOptimization (policy.h:74-86) */
	static SamplingParameters ApproximateGlobalOptimization()
	{
		SamplingParameters p;
		p.type = "regular"; p.base = "zero"; p.baseDirection = "unit"; p.radius = "maximum speed";
		p.angle = 360.0f; p.speedSamples = 11; p.angleSamples = 36; p.includeBaseAsSample = true;
		return p;
	}

	/* the XML attributes (crowdSimulator.cpp:344-373) of the set fields */
	std::vector<std::pair<std::string, std::string>> Attributes() const
	{
		auto check = [](const std::optional<std::string>& v, std::initializer_list<const char*> allowed,
		                const char* what) {
			if (!v) return;
			for (const char* a : allowed) if (*v == a) return;
			throw std::runtime_error(std::string("sampling ") + what + " '" + *v + "' is not allowed");
		};
		check(type, { "regular", "random" }, "type");
		check(base, { "zero", "current velocity" }, "base");
		check(baseDirection, { "unit", "current velocity", "preferred velocity" }, "base direction");
		check(radius, { "preferred speed", "maximum speed", "maximum acceleration" }, "radius");
		std::vector<std::pair<std::string, std::string>> a;
		if (type) a.emplace_back("SamplingType", *type);
		if (base) a.emplace_back("SamplingBase", *base);
		if (baseDirection) a.emplace_back("SamplingBaseDirection", *baseDirection);
		if (radius) a.emplace_back("SamplingRadius", *radius);
		if (angle) a.emplace_back("SamplingAngle", format_float(*angle));
		if (speedSamples) a.emplace_back("SpeedSamples", std::to_string(*speedSamples));
		if (angleSamples) a.emplace_back("AngleSamples", std::to_string(*angleSamples));
		if (randomSamples) a.emplace_back("RandomSamples", std::to_string(*randomSamples));
		if (includeBaseAsSample) a.emplace_back("IncludeBaseAsSample", *includeBaseAsSample ? "true" : "false");
		return a;
	}
};

/* One navigation policy (policy.h:127-181): an optimisation method, its
 * sampling parameters and up to four weighted cost functions. */
class Policy {
public:
	static constexpr int kMaxCostFunctions = 4;   /* per policy in this engine */

	Policy(int id, OptimizationMethod method, std::optional<SamplingParameters> sampling = std::nullopt)
		: id_(id), method_(method), sampling_(std::move(sampling))
	{
		if (sampling_ && method_ != OptimizationMethod::SAMPLING)
			throw std::runtime_error("sampling parameters are read for the sampling method only");
	}

	void setRelaxationTime(float t) { relax_ = t; }
	void setContactForceScale(float s) { contact_ = s; }
	int id() const { return id_; }

	/* Policy::AddCostFunction (policy.cpp:143-149): a registered cost
	 * function, its own parameters (the attributes its parseParameters reads),
	 * its range and weight */
	Policy& AddCostFunction(const std::string& name, const std::map<std::string, float>& params = {},
	                        std::optional<float> range = std::nullopt, std::optional<float> coeff = std::nullopt)
	{
		if ((int)costs_.size() == kMaxCostFunctions)
			throw std::runtime_error("more than 4 cost functions in a policy");
		if (!IsRegistered(name)) throw std::runtime_error("cost function '" + name + "' is not registered in this engine");
		std::vector<std::pair<std::string, std::string>> a;
		if (coeff) a.emplace_back("coeff", format_float(*coeff));
		if (range) a.emplace_back("range", format_float(*range));
		for (const auto& kv : params) a.emplace_back(kv.first, format_float(kv.second));
		costs_.emplace_back(name, std::move(a));
		return *this;
	}

	/* the <Policy> element */
	std::string ToXML() const
	{
		if (costs_.empty()) throw std::runtime_error("policy " + std::to_string(id_) + " needs a cost function");
		std::string s = "<Policy id=\"" + std::to_string(id_) + "\" OptimizationMethod=\"" + to_string(method_) + "\"";
		if (sampling_)
			for (const auto& kv : sampling_->Attributes()) s += " " + kv.first + "=\"" + kv.second + "\"";
		if (relax_) s += " RelaxationTime=\"" + format_float(*relax_) + "\"";
		if (contact_) s += " ContactForceScale=\"" + format_float(*contact_) + "\"";
		s += ">";
		for (const auto& c : costs_) {
			s += "<costfunction name=\"" + c.first + "\"";
			for (const auto& kv : c.second) s += " " + kv.first + "=\"" + kv.second + "\"";
			s += "/>";
		}
		return s + "</Policy>";
	}

	/* the registered cost-function names (CostFunctionFactory, plugins included) */
	static std::vector<std::string> RegisteredCostFunctions()
	{
		int n = 0;
		if (umans_cost_functions(nullptr, 0, &n) != UMANS_OK) throw std::runtime_error(umans_last_error(nullptr));
		std::vector<const char*> names((size_t)n);
		if (n > 0 && umans_cost_functions(names.data(), n, &n) != UMANS_OK)
			throw std::runtime_error(umans_last_error(nullptr));
		return std::vector<std::string>(names.begin(), names.end());
	}
	static bool IsRegistered(const std::string& name)
	{
		for (const auto& r : RegisteredCostFunctions()) if (r == name) return true;
		return false;
	}

private:
	int id_;
	OptimizationMethod method_;
	std::optional<SamplingParameters> sampling_;
	std::optional<float> relax_, contact_;
	std::vector<std::pair<std::string, std::vector<std::pair<std::string, std::string>>>> costs_;
};

/* WorldInfinite / WorldToric (worldInfinite.h, worldToric.h) */
enum class WorldType { Infinite, Toric };

struct Vec2 { float x, y; };

/* One agent as the scenario format describes it (crowdSimulator.cpp:
 * 424-510): position, goal, radius, preferred and maximum speed, policy, and
 * optionally a start time and removal at the goal. */
struct AgentSpec {
	Vec2 pos{ 0, 0 }, goal{ 0, 0 };
	float radius = 0.3f, prefSpeed = 1.3f, maxSpeed = 1.8f;
	int policy = 0;
	float startTime = 0;
	bool removeAtGoal = false;
};

/* A world with its time step, policies, agents and obstacles, written as
 * one scenario file. */
class World {
public:
	World(WorldType type, float dt, float width = 0, float height = 0) : type_(type), dt_(dt), w_(width), h_(height)
	{
		if (!(dt > 0)) throw std::runtime_error("the time step must be positive");
		if (type == WorldType::Toric && !(width > 0 && height > 0))
			throw std::runtime_error("a toric world needs a positive width and height");
	}
	void setEndTime(float t) { end_ = t; }
	void AddPolicy(const Policy& p) { policies_.push_back(p.ToXML()); }
	/* WorldBase::AddAgent (worldBase.cpp:161-186) */
	void AddAgent(Vec2 pos, Vec2 goal, int policy = 0)
	{
		AgentSpec a;
		a.pos = pos; a.goal = goal; a.policy = policy;
		agents_.push_back(a);
	}
	void AddAgent(const AgentSpec& a) { agents_.push_back(a); }
	/* WorldBase::AddObstacle (worldBase.cpp:239-242): a closed polygon */
	void AddObstacle(const std::vector<Vec2>& polygon) { obstacles_.push_back(polygon); }

	std::string ToXML() const
	{
		std::string s = "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n<Simulation delta_time=\"" + format_float(dt_) + "\"";
		if (end_) s += " end_time=\"" + format_float(*end_) + "\"";
		s += ">\n";
		std::string obs;
		if (!obstacles_.empty()) {
			obs = "<Obstacles>";
			for (const auto& poly : obstacles_) {
				obs += "<Obstacle>";
				for (const auto& p : poly) obs += "<Point x=\"" + format_float(p.x) + "\" y=\"" + format_float(p.y) + "\"/>";
				obs += "</Obstacle>";
			}
			obs += "</Obstacles>";
		}
		if (type_ == WorldType::Toric)
			s += "<World type=\"Toric\" width=\"" + format_float(w_) + "\" height=\"" + format_float(h_) + "\">" + obs + "</World>\n";
		else
			s += "<World type=\"Infinite\">" + obs + "</World>\n";
		s += "<Policies>\n";
		for (const auto& p : policies_) s += p + "\n";
		s += "</Policies>\n<Agents>\n";
		for (const auto& a : agents_) {
			s += "<Agent rad=\"" + format_float(a.radius) + "\" pref_speed=\"" + format_float(a.prefSpeed) +
			     "\" max_speed=\"" + format_float(a.maxSpeed) + "\"";
			if (a.startTime != 0) s += " start_time=\"" + format_float(a.startTime) + "\"";
			if (a.removeAtGoal) s += " remove_at_goal=\"true\"";
			s += "><pos x=\"" + format_float(a.pos.x) + "\" y=\"" + format_float(a.pos.y) + "\"/><goal x=\"" +
			     format_float(a.goal.x) + "\" y=\"" + format_float(a.goal.y) + "\"/><Policy id=\"" +
			     std::to_string(a.policy) + "\"/></Agent>\n";
		}
		return s + "</Agents>\n</Simulation>\n";
	}

	/* writes the scenario file; returns its path */
	std::string Write(const std::string& path) const
	{
		std::ofstream f(path);
		if (!f) throw std::runtime_error("cannot write " + path);
		f << ToXML();
		if (!f) throw std::runtime_error("cannot write " + path);
		return path;
	}

private:
	WorldType type_;
	float dt_, w_, h_;
	std::optional<float> end_;
	std::vector<std::string> policies_;
	std::vector<AgentSpec> agents_;
	std::vector<std::vector<Vec2>> obstacles_;
};

/* A simulation on the GPU made from a scenario file (umans_create); owns the
 * handle.  Needs a CUDA device. */
class Simulation {
public:
	explicit Simulation(const std::string& scenario_file)
	{
		if (umans_create(scenario_file.c_str(), &h_) != UMANS_OK) throw std::runtime_error(umans_last_error(nullptr));
	}
	~Simulation() { if (h_) umans_destroy(h_); }
	Simulation(const Simulation&) = delete;
	Simulation& operator=(const Simulation&) = delete;

	void Step(int n = 1) { check(umans_step(h_, n)); }
	int NumAgents() const
	{
		int n = 0;
		check(umans_num_agents(h_, &n));
		return n;
	}
	/* ids and positions, list order */
	void GetPositions(std::vector<int>& ids, std::vector<Vec2>& pos) const
	{
		const int n = NumAgents();
		ids.resize((size_t)n);
		pos.resize((size_t)n);
		check(umans_get_state(h_, ids.data(), &pos.data()->x, nullptr, nullptr, n));
	}
	umans_sim* handle() const { return h_; }

private:
	void check(int rc) const { if (rc != UMANS_OK) throw std::runtime_error(umans_last_error(h_)); }
	umans_sim* h_ = nullptr;
};

}  // namespace umans

#endif /* UMANS_GB300_HPP */
