// Host program of the zeno-host test: the MPM node plugin loaded into a real
// zeno core.  Prints, on lines that start with "ZSMPM_HOST ", (1) one JSON
// object with the descriptors of every node class the session holds, in the
// form of zsn_descriptors_json, and (2) the material ConfigConstitutiveModel
// makes, run through zeno's own Graph::addNode / setNodeInput / applyNodes
// with a "params" DictObject, one JSON object per line.
#include <zeno/core/Graph.h>
#include <zeno/core/INode.h>
#include <zeno/core/Session.h>
#include <zeno/types/DictObject.h>
#include <zeno/types/NumericObject.h>
#include <zeno/types/StringObject.h>
#include <zsmpm.h>

#include <cstdio>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>

namespace zeno {
bool zsmodel_material(const zany &obj, mpm_material *mat, float *volume);
}

namespace {

std::string esc(const std::string &s) {
  std::string o;
  for (char c : s) {
    if (c == '"' || c == '\\') {
      o += '\\';
      o += c;
    } else if ((unsigned char)c < 0x20) {
      char buf[8];
      std::snprintf(buf, sizeof buf, "\\u%04x", (unsigned)(unsigned char)c);
      o += buf;
    } else {
      o += c;
    }
  }
  return o;
}

template <class V> void sockets(std::ostringstream &os, const V &v) {
  os << "[";
  for (size_t i = 0; i < v.size(); ++i)
    os << (i ? "," : "") << "[\"" << esc(v[i].type) << "\",\"" << esc(v[i].name) << "\",\""
       << esc(v[i].defl) << "\"]";
  os << "]";
}

zeno::zany num(float v) { return std::make_shared<zeno::NumericObject>(zeno::NumericValue(v)); }
zeno::zany str(const std::string &v) {
  auto s = std::make_shared<zeno::StringObject>();
  s->set(v);
  return s;
}

void config_model(const char *type, const char *plasticity, float fa) {
  auto g = zeno::getSession().createGraph();
  g->addNode("ConfigConstitutiveModel", "m");
  g->setNodeInput("m", "dx", num(1.0f / 256));
  g->setNodeInput("m", "ppc", num(8.0f));
  g->setNodeInput("m", "density", num(1000.0f));
  g->setNodeInput("m", "type", str(type));
  g->setNodeInput("m", "aniso", str("none"));
  g->setNodeInput("m", "plasticity", str(plasticity));
  g->setNodeInput("m", "E", num(1e5f));
  g->setNodeInput("m", "nu", num(0.3f));
  if (fa > 0.0f) {
    auto d = std::make_shared<zeno::DictObject>();
    d->lut["friction_angle"] = num(fa);
    g->setNodeInput("m", "params", d);
  }
  g->applyNodes({"m"});
  mpm_material mat{};
  float vol = 0.0f;
  const bool ok = zeno::zsmodel_material(g->getNodeOutput("m", "ZSModel"), &mat, &vol);
  std::printf("ZSMPM_HOST {\"model\":%d,\"type\":%d,\"plasticity\":%d,\"friction_angle_deg\":%.9g,"
              "\"volume\":%.9g}\n",
              ok ? 1 : 0, mat.type, mat.plasticity, mat.friction_angle_deg, vol);
}

}  // namespace

int main() {
  auto &sess = zeno::getSession();
  std::ostringstream os;
  os << "{";
  bool first = true;
  for (const auto &[name, cls] : sess.nodeClasses) {
    const zeno::Descriptor &d = *cls->desc;
    os << (first ? "" : ",") << "\"" << esc(name) << "\":{\"inputs\":";
    first = false;
    sockets(os, d.inputs);
    os << ",\"outputs\":";
    sockets(os, d.outputs);
    os << ",\"params\":";
    sockets(os, d.params);
    os << ",\"categories\":[";
    for (size_t i = 0; i < d.categories.size(); ++i)
      os << (i ? "," : "") << "\"" << esc(d.categories[i]) << "\"";
    os << "]}";
  }
  os << "}";
  std::cout << "ZSMPM_HOST " << os.str() << "\n";
  config_model("stvk", "nadp", 30.0f);
  config_model("stvk", "nadp", 0.0f);
  config_model("snhk", "none", 0.0f);
  return 0;
}
