#include "xml.hpp"

#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace umans {

const char* XmlElement::attr(const char* key) const
{
	for (const auto& a : attrs)
		if (a.first == key) return a.second.c_str();
	return nullptr;
}

static bool skip_ws_all(const char* s)
{
	while (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r') ++s;
	return *s == 0;
}

bool XmlElement::query_float(const char* key, float* out) const
{
	const char* v = attr(key);
	if (!v) return false;
	char* end = nullptr;
	errno = 0;
	float f = std::strtof(v, &end);   // correctly rounded, like tinyxml2's "%f" scan
	if (end == v) return false;
	*out = f;
	return true;
}

bool XmlElement::query_int(const char* key, int* out) const
{
	const char* v = attr(key);
	if (!v) return false;
	char* end = nullptr;
	long x = std::strtol(v, &end, 10);
	if (end == v) return false;
	*out = (int)x;
	return true;
}

bool XmlElement::query_bool(const char* key, bool* out) const
{
	const char* v = attr(key);
	if (!v) return false;
	int i;
	char* end = nullptr;
	long x = std::strtol(v, &end, 10);
	if (end != v) { i = (int)x; *out = i != 0; return true; }
	std::string s(v);
	if (s == "true" || s == "True" || s == "TRUE") { *out = true; return true; }
	if (s == "false" || s == "False" || s == "FALSE") { *out = false; return true; }
	return false;
}

const XmlElement* XmlElement::first_child(const char* nm) const
{
	for (const auto& c : children)
		if (!nm || c->name == nm) return c.get();
	return nullptr;
}

const XmlElement* XmlElement::next_sibling(const XmlElement* child, const char* nm) const
{
	// from the child's own position (constant time per step of a sibling walk)
	size_t k = 0;
	if (child && child->index < children.size() && children[child->index].get() == child) k = child->index + 1;
	else {
		while (k < children.size() && children[k].get() != child) ++k;
		if (k == children.size()) return nullptr;
		++k;
	}
	for (; k < children.size(); ++k)
		if (!nm || children[k]->name == nm) return children[k].get();
	return nullptr;
}

namespace {

struct Parser {
	const std::string& t;
	size_t i = 0;
	std::string err;
	explicit Parser(const std::string& text) : t(text) {}

	bool eof() const { return i >= t.size(); }
	void ws() { while (!eof() && (t[i] == ' ' || t[i] == '\t' || t[i] == '\n' || t[i] == '\r')) ++i; }
	bool starts(const char* s) const { return t.compare(i, std::strlen(s), s) == 0; }

	bool skip_until(const char* s)
	{
		size_t p = t.find(s, i);
		if (p == std::string::npos) { err = std::string("unterminated construct, expected ") + s; return false; }
		i = p + std::strlen(s);
		return true;
	}

	static std::string unescape(const std::string& s)
	{
		std::string o;
		for (size_t k = 0; k < s.size(); ++k) {
			if (s[k] == '&') {
				size_t e = s.find(';', k);
				if (e != std::string::npos) {
					std::string ent = s.substr(k + 1, e - k - 1);
					if (ent == "lt") { o += '<'; k = e; continue; }
					if (ent == "gt") { o += '>'; k = e; continue; }
					if (ent == "amp") { o += '&'; k = e; continue; }
					if (ent == "quot") { o += '"'; k = e; continue; }
					if (ent == "apos") { o += '\''; k = e; continue; }
				}
			}
			o += s[k];
		}
		return o;
	}

	// skips comments, declarations, processing instructions and text
	bool misc()
	{
		for (;;) {
			ws();
			if (eof()) return true;
			if (starts("<!--")) { if (!skip_until("-->")) return false; continue; }
			if (starts("<?")) { if (!skip_until("?>")) return false; continue; }
			if (starts("<![CDATA[")) { if (!skip_until("]]>")) return false; continue; }
			if (starts("<!")) { if (!skip_until(">")) return false; continue; }
			if (t[i] != '<') { size_t p = t.find('<', i); i = (p == std::string::npos) ? t.size() : p; continue; }
			return true;
		}
	}

	bool name(std::string& out)
	{
		size_t s = i;
		while (!eof() && !std::strchr(" \t\r\n/>=", t[i])) ++i;
		out = t.substr(s, i - s);
		if (out.empty()) { err = "empty name"; return false; }
		return true;
	}

	bool element(XmlElement& e)
	{
		++i;   // '<'
		if (!name(e.name)) return false;
		for (;;) {
			ws();
			if (eof()) { err = "unexpected end in tag"; return false; }
			if (starts("/>")) { i += 2; return true; }
			if (t[i] == '>') { ++i; break; }
			std::string k;
			if (!name(k)) return false;
			ws();
			if (eof() || t[i] != '=') { err = "expected '=' after attribute " + k; return false; }
			++i;
			ws();
			if (eof() || (t[i] != '"' && t[i] != '\'')) { err = "expected quoted value"; return false; }
			char q = t[i++];
			size_t p = t.find(q, i);
			if (p == std::string::npos) { err = "unterminated attribute value"; return false; }
			e.attrs.emplace_back(k, unescape(t.substr(i, p - i)));
			i = p + 1;
		}
		for (;;) {
			if (!misc()) return false;
			if (eof()) { err = "missing closing tag for " + e.name; return false; }
			if (starts("</")) {
				i += 2;
				std::string nm;
				if (!name(nm)) return false;
				if (nm != e.name) { err = "mismatched closing tag " + nm + " for " + e.name; return false; }
				ws();
				if (eof() || t[i] != '>') { err = "malformed closing tag"; return false; }
				++i;
				return true;
			}
			auto c = std::make_unique<XmlElement>();
			if (!element(*c)) return false;
			c->index = e.children.size();
			e.children.push_back(std::move(c));
		}
	}
};

}  // namespace

bool XmlDocument::parse(const std::string& text)
{
	root = XmlElement();
	Parser p(text);
	for (;;) {
		if (!p.misc()) { error = p.err; return false; }
		if (p.eof()) break;
		auto c = std::make_unique<XmlElement>();
		if (!p.element(*c)) { error = p.err; return false; }
		c->index = root.children.size();
		root.children.push_back(std::move(c));
	}
	if (root.children.empty()) { error = "no element in document"; return false; }
	return true;
}

bool XmlDocument::load_file(const std::string& path)
{
	std::ifstream f(path, std::ios::binary);
	if (!f) { error = "cannot open " + path; return false; }
	std::stringstream ss;
	ss << f.rdbuf();
	return parse(ss.str());
}

}  // namespace umans
