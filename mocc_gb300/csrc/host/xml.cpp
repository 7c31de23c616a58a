#include "xml.hpp"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "geom.hpp"

namespace mocgpu {

const XmlNode *XmlNode::child(const std::string &n) const
{
    for (const auto &c : children)
        if (c->name == n) return c.get();
    return nullptr;
}

std::vector<const XmlNode *> XmlNode::children_named(const std::string &n) const
{
    std::vector<const XmlNode *> out;
    for (const auto &c : children)
        if (c->name == n) out.push_back(c.get());
    return out;
}

bool XmlNode::has_attr(const std::string &n) const
{
    for (const auto &a : attrs)
        if (a.first == n) return true;
    return false;
}

std::string XmlNode::attr(const std::string &n, const std::string &dflt) const
{
    for (const auto &a : attrs)
        if (a.first == n) return a.second;
    return dflt;
}

double XmlNode::attr_double(const std::string &n, double dflt) const
{
    if (!has_attr(n)) return dflt;
    std::string v = attr(n);
    char *end = nullptr;
    double d = std::strtod(v.c_str(), &end);
    if (end == v.c_str()) return dflt;
    return d;
}

int XmlNode::attr_int(const std::string &n, int dflt) const
{
    if (!has_attr(n)) return dflt;
    std::string v = attr(n);
    char *end = nullptr;
    long d = std::strtol(v.c_str(), &end, 10);
    if (end == v.c_str()) return dflt;
    return (int)d;
}

bool XmlNode::attr_bool(const std::string &n, bool dflt) const
{
    if (!has_attr(n)) return dflt;
    std::string v = attr(n);
    if (v.empty()) return dflt;
    // pugixml as_bool: true when the first character is 1, t, T, y or Y.
    char c = v[0];
    return c == '1' || c == 't' || c == 'T' || c == 'y' || c == 'Y';
}

void XmlNode::set_attr(const std::string &n, const std::string &v)
{
    for (auto &a : attrs)
        if (a.first == n) {
            a.second = v;
            return;
        }
    attrs.emplace_back(n, v);
}

namespace {

struct Parser {
    const std::string &s;
    size_t i = 0;
    explicit Parser(const std::string &src) : s(src) {}

    [[noreturn]] void fail(const std::string &what)
    {
        MOCGPU_THROW(2, "XML parse error at offset " + std::to_string(i) + ": " + what);
    }
    bool starts(const char *p) const { return s.compare(i, std::char_traits<char>::length(p), p) == 0; }
    void skip_ws()
    {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    static std::string decode(const std::string &t)
    {
        std::string out;
        out.reserve(t.size());
        for (size_t k = 0; k < t.size(); k++) {
            if (t[k] == '&') {
                size_t e = t.find(';', k);
                if (e != std::string::npos) {
                    std::string ent = t.substr(k + 1, e - k - 1);
                    if (ent == "lt") out += '<';
                    else if (ent == "gt") out += '>';
                    else if (ent == "amp") out += '&';
                    else if (ent == "quot") out += '"';
                    else if (ent == "apos") out += '\'';
                    else out += t.substr(k, e - k + 1);
                    k = e;
                    continue;
                }
            }
            out += t[k];
        }
        return out;
    }
    void skip_misc()
    {
        while (true) {
            skip_ws();
            if (starts("<!--")) {
                size_t e = s.find("-->", i);
                if (e == std::string::npos) fail("unterminated comment");
                i = e + 3;
            } else if (starts("<?")) {
                size_t e = s.find("?>", i);
                if (e == std::string::npos) fail("unterminated declaration");
                i = e + 2;
            } else if (starts("<!")) {
                size_t e = s.find('>', i);
                if (e == std::string::npos) fail("unterminated markup");
                i = e + 1;
            } else {
                return;
            }
        }
    }
    std::string name()
    {
        size_t b = i;
        while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' ||
                                s[i] == ':' || s[i] == '.'))
            i++;
        if (b == i) fail("expected a name");
        return s.substr(b, i - b);
    }
    std::unique_ptr<XmlNode> element()
    {
        if (s[i] != '<') fail("expected '<'");
        i++;
        auto node = std::make_unique<XmlNode>();
        node->name = name();
        while (true) {
            skip_ws();
            if (i >= s.size()) fail("unterminated tag");
            if (s[i] == '/') {
                if (i + 1 >= s.size() || s[i + 1] != '>') fail("bad self-closing tag");
                i += 2;
                return node;
            }
            if (s[i] == '>') {
                i++;
                break;
            }
            std::string an = name();
            skip_ws();
            if (i >= s.size() || s[i] != '=') fail("expected '=' after attribute " + an);
            i++;
            skip_ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) fail("expected quoted value");
            char q = s[i++];
            size_t e = s.find(q, i);
            if (e == std::string::npos) fail("unterminated attribute value");
            node->attrs.emplace_back(an, decode(s.substr(i, e - i)));
            i = e + 1;
        }
        // content
        while (true) {
            if (i >= s.size()) fail("unterminated element " + node->name);
            if (starts("</")) {
                i += 2;
                std::string en = name();
                if (en != node->name) fail("mismatched close tag " + en + " for " + node->name);
                skip_ws();
                if (i >= s.size() || s[i] != '>') fail("expected '>'");
                i++;
                return node;
            }
            if (starts("<!--")) {
                size_t e = s.find("-->", i);
                if (e == std::string::npos) fail("unterminated comment");
                i = e + 3;
                continue;
            }
            if (starts("<![CDATA[")) {
                size_t e = s.find("]]>", i);
                if (e == std::string::npos) fail("unterminated CDATA");
                node->text += s.substr(i + 9, e - i - 9);
                i = e + 3;
                continue;
            }
            if (s[i] == '<') {
                node->children.push_back(element());
                continue;
            }
            size_t e = s.find('<', i);
            if (e == std::string::npos) fail("unterminated text");
            node->text += decode(s.substr(i, e - i));
            i = e;
        }
    }
};

} // namespace

std::unique_ptr<XmlNode> parse_xml(const std::string &text)
{
    Parser p(text);
    auto doc = std::make_unique<XmlNode>();
    doc->name = "#document";
    while (true) {
        p.skip_misc();
        if (p.i >= text.size()) break;
        if (text[p.i] != '<') p.fail("text outside of an element");
        doc->children.push_back(p.element());
    }
    return doc;
}

std::string read_file(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) MOCGPU_THROW(3, "cannot open file: " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::string sanitize(std::string s)
{
    s.erase(std::remove_if(s.begin(), s.end(), [](unsigned char c) { return std::isspace(c); }), s.end());
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
    return s;
}

template <> std::vector<int> explode<int>(const std::string &s)
{
    std::vector<int> out;
    std::istringstream in(s);
    std::string tok;
    while (in >> tok) {
        char *end = nullptr;
        long v = std::strtol(tok.c_str(), &end, 10);
        if (*end != '\0') MOCGPU_THROW(2, "bad integer in list: " + tok);
        out.push_back((int)v);
    }
    return out;
}

template <> std::vector<double> explode<double>(const std::string &s)
{
    std::vector<double> out;
    std::istringstream in(s);
    std::string tok;
    while (in >> tok) {
        char *end = nullptr;
        double v = std::strtod(tok.c_str(), &end);
        if (*end != '\0') MOCGPU_THROW(2, "bad number in list: " + tok);
        out.push_back(v);
    }
    return out;
}

} // namespace mocgpu
