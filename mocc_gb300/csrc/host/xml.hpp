// Minimal XML reader for MOCC's input subset (elements, attributes, text,
// comments). MOCC parses its input with pugixml; its documents have several
// top-level elements, so the parser returns a synthetic document node whose
// children are the top-level elements (the same view pugixml gives).
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace mocgpu {

struct XmlNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::string text; // concatenated character data of this element
    std::vector<std::unique_ptr<XmlNode>> children;

    const XmlNode *child(const std::string &n) const;
    std::vector<const XmlNode *> children_named(const std::string &n) const;
    bool has_attr(const std::string &n) const;
    std::string attr(const std::string &n, const std::string &dflt = "") const;
    double attr_double(const std::string &n, double dflt) const;
    int attr_int(const std::string &n, int dflt) const;
    bool attr_bool(const std::string &n, bool dflt) const;
    void set_attr(const std::string &n, const std::string &v);
};

// Parses a document; throws mocgpu::Error on malformed input.
std::unique_ptr<XmlNode> parse_xml(const std::string &text);
std::string read_file(const std::string &path);

// Lower-case and strip whitespace (MOCC's sanitize()).
std::string sanitize(std::string s);

template <typename T> std::vector<T> explode(const std::string &s);

} // namespace mocgpu
