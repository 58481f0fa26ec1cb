/* Test-infrastructure stand-in for the vendored yaml-cpp 0.2 API used by the
 * reference's io/parseDomainFile.cu and io/parseBodiesFile.cu.
 *
 * The document is read as JSON (tests write each case description as JSON next
 * to the YAML they give the product), which has the same tree shape.  Like
 * yaml-cpp 0.2, looking up a missing key or index throws, and `node >> x`
 * converts the scalar text with a stringstream (bools from true/false). */
#pragma once
#include <istream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace YAML {
class Node {
  public:
    enum Kind { Null, Scalar, Seq, Map } kind = Null;
    std::string text;
    std::vector<std::shared_ptr<Node>> items;
    std::map<std::string, std::shared_ptr<Node>> keys;

    const Node &operator[](const std::string &k) const {
        auto it = keys.find(k);
        if (kind != Map || it == keys.end()) throw std::runtime_error("key not found: " + k);
        return *it->second;
    }
    const Node &operator[](const char *k) const { return (*this)[std::string(k)]; }
    const Node &operator[](int i) const {
        if (kind != Seq || i < 0 || i >= (int)items.size()) throw std::runtime_error("bad index");
        return *items[i];
    }
    const Node &operator[](unsigned i) const { return (*this)[(int)i]; }
    unsigned size() const { return kind == Seq ? items.size() : kind == Map ? keys.size() : 0; }
};

inline void ref_skip(const std::string &s, size_t &p) {
    while (p < s.size() && (s[p] == ' ' || s[p] == '\n' || s[p] == '\t' || s[p] == '\r' || s[p] == ',' ||
                            s[p] == ':'))
        ++p;
}
inline std::shared_ptr<Node> ref_parse(const std::string &s, size_t &p) {
    ref_skip(s, p);
    auto n = std::make_shared<Node>();
    if (s[p] == '{') {
        n->kind = Node::Map;
        ++p;
        for (;;) {
            ref_skip(s, p);
            if (s[p] == '}') { ++p; break; }
            auto k = ref_parse(s, p);
            auto v = ref_parse(s, p);
            n->keys[k->text] = v;
        }
    } else if (s[p] == '[') {
        n->kind = Node::Seq;
        ++p;
        for (;;) {
            ref_skip(s, p);
            if (s[p] == ']') { ++p; break; }
            n->items.push_back(ref_parse(s, p));
        }
    } else if (s[p] == '"') {
        n->kind = Node::Scalar;
        size_t q = s.find('"', p + 1);
        n->text = s.substr(p + 1, q - p - 1);
        p = q + 1;
    } else {
        n->kind = Node::Scalar;
        size_t q = p;
        while (q < s.size() && s[q] != ',' && s[q] != ']' && s[q] != '}' && s[q] != '\n' && s[q] != ' ') ++q;
        n->text = s.substr(p, q - p);
        p = q;
    }
    return n;
}

class Parser {
    std::string src;
  public:
    explicit Parser(std::istream &in) {
        std::stringstream ss;
        ss << in.rdbuf();
        src = ss.str();
    }
    bool GetNextDocument(Node &doc) {
        size_t p = 0;
        doc = *ref_parse(src, p);
        return true;
    }
};

template <class T>
inline void operator>>(const Node &n, T &v) {
    if (n.kind != Node::Scalar) throw std::runtime_error("not a scalar");
    std::stringstream ss(n.text);
    ss >> v;
}
inline void operator>>(const Node &n, bool &v) {
    if (n.kind != Node::Scalar) throw std::runtime_error("not a scalar");
    v = (n.text == "true" || n.text == "True" || n.text == "1");
}
inline void operator>>(const Node &n, std::string &v) {
    if (n.kind != Node::Scalar) throw std::runtime_error("not a scalar");
    v = n.text;
}
}  // namespace YAML
