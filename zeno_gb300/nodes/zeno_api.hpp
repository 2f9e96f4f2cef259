// Host-side mirror of the zeno node-plugin interface the MPM nodes are
// written against, so the node wrappers compile and run headless without
// the rest of zeno:
//   IObject / zany                 zeno/include/zeno/core/IObject.h:89
//   NumericObject, DictObject,
//   PrimitiveObject                zeno/include/zeno/types/*.h
//   INode (get_input, get_input2, has_input, set_output, get_param)
//                                  zeno/include/zeno/core/INode.h:23-127
//   Descriptor + ZENDEFNODE        zeno/include/zeno/core/Descriptor.h, defNode.h:16-34
//   Graph (addNode, setNodeInput, bindNodeInput, applyNodes, getNodeOutput)
//                                  zeno/src/core/Graph.cpp:81-112
// Names, argument meaning and error behaviour (exceptions carrying the
// socket and node name) follow the reference; the object model is reduced to
// what the MPM nodes exchange.  Inside zeno the node file includes zeno's
// own headers instead of this one.
#pragma once

#include <array>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

namespace zeno {

using vec3f = std::array<float, 3>;
using vec3i = std::array<int, 3>;
using vec2i = std::array<int, 2>;
using vec4i = std::array<int, 4>;

struct IObject {
  virtual ~IObject() = default;
};
using zany = std::shared_ptr<IObject>;

// NumericObject: int / float / vec3f (zeno/include/zeno/types/NumericObject.h)
struct NumericObject : IObject {
  std::variant<int, float, vec3f> value = 0.0f;
  NumericObject() = default;
  template <class T> explicit NumericObject(T v) : value(v) {}
  template <class T> T get() const {
    if constexpr (std::is_same_v<T, vec3f>) {
      if (auto p = std::get_if<vec3f>(&value)) return *p;
      throw std::runtime_error("NumericObject does not hold a vec3f");
    } else {
      if (auto p = std::get_if<float>(&value)) return static_cast<T>(*p);
      if (auto p = std::get_if<int>(&value)) return static_cast<T>(*p);
      throw std::runtime_error("NumericObject does not hold a scalar");
    }
  }
  template <class T> void set(T v) { value = v; }
};

// DictObject: named objects (zeno/include/zeno/types/DictObject.h:11-31);
// ConfigConstitutiveModel's "params" holds NumericObjects by key
struct DictObject : IObject {
  std::map<std::string, zany> lut;
};

struct StringObject : IObject {
  std::string value;
  StringObject() = default;
  explicit StringObject(std::string v) : value(std::move(v)) {}
};

// PrimitiveObject: vertex positions plus named vertex attributes
// (zeno/include/zeno/types/PrimitiveObject.h); "pos" is the position.
struct PrimitiveObject : IObject {
  std::map<std::string, std::vector<vec3f>> attrs3;
  std::map<std::string, std::vector<float>> attrs1;
  std::vector<vec3i> tris;  // triangle vertex indices
  std::vector<vec2i> lines; // segment vertex indices
  std::vector<vec4i> quads; // tetrahedron vertex indices
  std::map<std::string, std::vector<vec3f>> tri_attrs3;  // per-triangle attributes
  std::map<std::string, std::vector<float>> tri_attrs1;
  std::vector<vec3f> &verts() { return attrs3["pos"]; }
  size_t size() const {
    auto it = attrs3.find("pos");
    return it == attrs3.end() ? 0 : it->second.size();
  }
  bool has_attr(const std::string &k) const { return attrs3.count(k) || attrs1.count(k); }
};

struct SocketDescriptor {
  std::string type, name, defl;
  SocketDescriptor(const char *n) : name(n) {}  // NOLINT: brace-init of descriptors
  SocketDescriptor(std::string t, std::string n, std::string d = "")
      : type(std::move(t)), name(std::move(n)), defl(std::move(d)) {}
};
using ParamDescriptor = SocketDescriptor;

struct Descriptor {
  std::vector<SocketDescriptor> inputs, outputs;
  std::vector<ParamDescriptor> params;
  std::vector<std::string> categories;
};

struct INode;
struct NodeClass {
  std::function<std::unique_ptr<INode>()> ctor;
  Descriptor desc;
};

inline std::map<std::string, NodeClass> &node_registry() {
  static std::map<std::string, NodeClass> r;
  return r;
}

namespace detail {
inline float to_float(const std::string &s) { return std::stof(s); }
inline int to_int(const std::string &s) { return std::stoi(s); }
}  // namespace detail

struct INode {
  std::string myname;
  const NodeClass *nodeClass = nullptr;
  std::map<std::string, zany> inputs;
  std::map<std::string, zany> outputs;

  virtual ~INode() = default;
  virtual void apply() = 0;

  bool has_input(const std::string &id) const { return inputs.count(id) && inputs.at(id); }
  zany get_input(const std::string &id) const {
    auto it = inputs.find(id);
    if (it == inputs.end() || !it->second)
      throw std::runtime_error("input socket `" + id + "` of node `" + myname +
                               "` is not connected");
    return it->second;
  }
  template <class T> std::shared_ptr<T> get_input(const std::string &id) const {
    auto p = std::dynamic_pointer_cast<T>(get_input(id));
    if (!p)
      throw std::runtime_error("input socket `" + id + "` of node `" + myname +
                               "` has an object of the wrong type");
    return p;
  }
  template <class T> bool has_input(const std::string &id) const {
    return has_input(id) && std::dynamic_pointer_cast<T>(inputs.at(id)) != nullptr;
  }
  void set_output(const std::string &id, zany obj) { outputs[id] = std::move(obj); }

  // literal inputs: the connected object, else the descriptor default
  template <class T> T get_input2(const std::string &id) const {
    if (has_input(id)) {
      auto o = inputs.at(id);
      if constexpr (std::is_same_v<T, std::string>) {
        if (auto s = std::dynamic_pointer_cast<StringObject>(o)) return s->value;
      } else {
        if (auto n = std::dynamic_pointer_cast<NumericObject>(o)) return n->get<T>();
      }
      throw std::runtime_error("input socket `" + id + "` of node `" + myname +
                               "` is not a literal of the expected type");
    }
    return defl<T>(id);
  }
  template <class T> T get_param(const std::string &id) const { return get_input2<T>(id + ":"); }

 private:
  template <class T> T defl(const std::string &id) const {
    const std::string key = (!id.empty() && id.back() == ':') ? id.substr(0, id.size() - 1) : id;
    const auto &d = nodeClass->desc;
    for (auto *list : {&d.inputs, &d.params})
      for (const auto &s : *list)
        if (s.name == key) {
          std::string v = s.defl;
          if constexpr (std::is_same_v<T, std::string>) {
            return v;
          } else if constexpr (std::is_same_v<T, float>) {
            return detail::to_float(v);
          } else if constexpr (std::is_same_v<T, int>) {
            return detail::to_int(v);
          } else {
            static_assert(sizeof(T) == 0, "unsupported literal type");
          }
        }
    throw std::runtime_error("no input or default for socket `" + key + "` of node `" + myname +
                             "`");
  }
};

template <class N> int defNodeClass(const char *name, Descriptor desc) {
  NodeClass c;
  c.ctor = [] { return std::unique_ptr<INode>(new N()); };
  c.desc = std::move(desc);
  node_registry()[name] = std::move(c);
  return 1;
}

#define ZENDEFNODE(Class, ...) \
  static int _zsmpm_def_##Class = ::zeno::defNodeClass<Class>(#Class, ::zeno::Descriptor __VA_ARGS__)

// Headless graph: nodes bound by sockets and evaluated on demand, each at
// most once per applyNodes() call (Graph::applyNode memoises per context).
struct Graph {
  struct Link {
    std::string node, socket;
  };
  struct Entry {
    std::unique_ptr<INode> node;
    std::map<std::string, zany> literals;
    std::map<std::string, Link> links;
  };
  std::map<std::string, Entry> nodes;
  // nodes evaluated once and then reused by later applyNodes() calls: the
  // setup nodes outside a BeginFor/EndFor loop body
  // (zeno/src/nodes/ControlNodes.cpp:46-112)
  std::set<std::string> once, done_once;
  void markOnce(const std::string &id) { once.insert(id); }

  void addNode(const std::string &cls, const std::string &id) {
    auto it = node_registry().find(cls);
    if (it == node_registry().end()) throw std::runtime_error("no node class named `" + cls + "`");
    Entry e;
    e.node = it->second.ctor();
    e.node->myname = id;
    e.node->nodeClass = &it->second;
    nodes[id] = std::move(e);
  }
  void setNodeInput(const std::string &id, const std::string &socket, zany obj) {
    entry(id).literals[socket] = std::move(obj);
  }
  void bindNodeInput(const std::string &dst, const std::string &dsock, const std::string &src,
                     const std::string &ssock) {
    entry(dst).links[dsock] = Link{src, ssock};
  }
  void applyNodes(const std::vector<std::string> &ids) {
    std::set<std::string> visited;
    for (const auto &id : ids) applyNode(id, visited);
  }
  zany getNodeOutput(const std::string &id, const std::string &socket) {
    auto &o = entry(id).node->outputs;
    auto it = o.find(socket);
    if (it == o.end())
      throw std::runtime_error("node `" + id + "` has no output `" + socket + "`");
    return it->second;
  }

 private:
  Entry &entry(const std::string &id) {
    auto it = nodes.find(id);
    if (it == nodes.end()) throw std::runtime_error("no node `" + id + "` in the graph");
    return it->second;
  }
  void applyNode(const std::string &id, std::set<std::string> &visited) {
    if (visited.count(id)) return;
    visited.insert(id);
    if (once.count(id) && done_once.count(id)) return;
    if (once.count(id)) done_once.insert(id);
    Entry &e = entry(id);
    e.node->inputs = e.literals;
    for (auto &[sock, link] : e.links) {
      applyNode(link.node, visited);
      e.node->inputs[sock] = getNodeOutput(link.node, link.socket);
    }
    e.node->outputs.clear();
    e.node->apply();
  }
};

}  // namespace zeno
