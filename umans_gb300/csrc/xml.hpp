// Minimal XML reader for UMANS scenario files.
//
// Scenario, policy and agent files are small element trees with attributes;
// text content is never read.  The reader accepts what the reference's
// tinyxml2 accepts in the shipped examples: several top-level elements in one
// file (examples/agents/1to10-180Degrees.xml) and comments containing "--"
// (examples/agents/25to25-Formation-90Degrees.xml).
#pragma once
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace umans {

struct XmlElement {
	std::string name;
	std::vector<std::pair<std::string, std::string>> attrs;
	std::vector<std::unique_ptr<XmlElement>> children;
	size_t index = 0;   // position among its parent's children

	const char* attr(const char* key) const;
	// tinyxml2-style typed queries: true when the attribute exists and parses
	bool query_float(const char* key, float* out) const;
	bool query_int(const char* key, int* out) const;
	bool query_bool(const char* key, bool* out) const;

	const XmlElement* first_child(const char* name = nullptr) const;
	// next sibling of `child` among this element's children, optionally by name
	const XmlElement* next_sibling(const XmlElement* child, const char* name = nullptr) const;
};

struct XmlDocument {
	XmlElement root;   // synthetic: its children are the top-level elements
	std::string error;
	bool load_file(const std::string& path);
	bool parse(const std::string& text);
};

}  // namespace umans
