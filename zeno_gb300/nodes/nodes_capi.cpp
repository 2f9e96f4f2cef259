// Test entry points of the node layer (libzsmpm_nodes.so):
//  * the registered node descriptors as JSON, to check names, sockets and
//    defaults against the reference's ZENDEFNODE declarations;
//  * one headless run of the reference substep graph built from those nodes
//    with Graph::addNode / setNodeInput / bindNodeInput / applyNodes, the
//    way a zeno graph wires them (the loop body is re-applied per substep,
//    the setup nodes are evaluated once).
#include <zsmpm.h>

#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>

#include "zeno_api.hpp"

namespace zeno {
bool zsmodel_material(const zany &obj, mpm_material *mat, float *volume);
}

namespace {

std::string esc(const std::string &s) {
  std::string o;
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
  }
  return o;
}

void sockets(std::ostringstream &os, const std::vector<zeno::SocketDescriptor> &v) {
  os << "[";
  for (size_t i = 0; i < v.size(); ++i) {
    if (i) os << ",";
    os << "[\"" << esc(v[i].type) << "\",\"" << esc(v[i].name) << "\",\"" << esc(v[i].defl)
       << "\"]";
  }
  os << "]";
}

int32_t copy_out(const std::string &s, char *buf, int64_t cap) {
  if (!buf || cap <= 0) return -1;
  const size_t n = std::min<size_t>(s.size(), (size_t)cap - 1);
  std::memcpy(buf, s.data(), n);
  buf[n] = 0;
  return (int32_t)s.size();
}

}  // namespace

extern "C" {

// JSON object {node name: {inputs, outputs, params, categories}}; returns the
// full length (the buffer holds cap - 1 characters at most).
int32_t zsn_descriptors_json(char *buf, int64_t cap) {
  std::ostringstream os;
  os << "{";
  bool first = true;
  for (const auto &[name, cls] : zeno::node_registry()) {
    if (!first) os << ",";
    first = false;
    os << "\"" << esc(name) << "\":{\"inputs\":";
    sockets(os, cls.desc.inputs);
    os << ",\"outputs\":";
    sockets(os, cls.desc.outputs);
    os << ",\"params\":";
    sockets(os, cls.desc.params);
    os << ",\"categories\":[";
    for (size_t i = 0; i < cls.desc.categories.size(); ++i)
      os << (i ? "," : "") << "\"" << esc(cls.desc.categories[i]) << "\"";
    os << "]}";
  }
  os << "}";
  return copy_out(os.str(), buf, cap);
}

// One ConfigConstitutiveModel node (dx, ppc, density, type, aniso,
// plasticity, E, nu and a "params" dict given as "key=value;key=value")
// applied through the graph; returns the material and particle volume its
// ZSModel carries, or -1 with the node's error text in err.
int32_t zsn_config_model(float dx, float ppc, float density, const char *type, const char *aniso,
                         const char *plasticity, float E, float nu, const char *params,
                         mpm_material *out, float *out_volume, char *err, int64_t err_cap) {
  using namespace zeno;
  try {
    Graph g;
    auto num = [](float v) { return std::make_shared<NumericObject>(v); };
    auto str = [](const char *v) { return std::make_shared<StringObject>(v); };
    g.addNode("ConfigConstitutiveModel", "model");
    g.setNodeInput("model", "dx", num(dx));
    g.setNodeInput("model", "ppc", num(ppc));
    g.setNodeInput("model", "density", num(density));
    g.setNodeInput("model", "type", str(type));
    g.setNodeInput("model", "aniso", str(aniso));
    g.setNodeInput("model", "plasticity", str(plasticity));
    g.setNodeInput("model", "E", num(E));
    g.setNodeInput("model", "nu", num(nu));
    if (params && params[0]) {
      auto dict = std::make_shared<DictObject>();
      std::istringstream ps(params);
      std::string item;
      while (std::getline(ps, item, ';')) {
        const size_t eq = item.find('=');
        if (eq == std::string::npos) continue;
        dict->lut[item.substr(0, eq)] = num(std::stof(item.substr(eq + 1)));
      }
      g.setNodeInput("model", "params", dict);
    }
    g.applyNodes({"model"});
    if (!zsmodel_material(g.getNodeOutput("model", "ZSModel"), out, out_volume))
      throw std::runtime_error("ConfigConstitutiveModel did not output a ZSModel");
    return 0;
  } catch (const std::exception &e) {
    copy_out(e.what(), err, err_cap);
    return -1;
  }
}

// Runs `substeps` substeps of one particle set through the node graph
// (fused = 0: the reference's node sequence per substep; fused = 1: one
// ZSMPMSubstep node) and returns x, v (n x 3) and the last MaxVelSqr.
int32_t zsn_run_graph(int32_t fused, int64_t n, const float *pos, const float *vel, float dx,
                      const char *type, const char *plasticity, float E, float nu,
                      float density, float ppc, const char *bc_type, int32_t bc_thickness,
                      float dt, float gravity, int32_t substeps, float *out_x, float *out_v,
                      float *out_max_vel_sqr, char *err, int64_t err_cap,
                      const char *ls_shape, const float *ls, const char *ls_type,
                      const char *transfer, int64_t cloth_nv, const float *cloth_x,
                      const float *cloth_v, int64_t cloth_nt, const int32_t *cloth_tris,
                      const float *cloth_params, float *cloth_out_x, float *cloth_out_v,
                      int64_t tracker_n, const float *tracker_x, float *tracker_out_x,
                      float *tracker_out_v, const char *write_path, const char *bending_type,
                      float bending_stiffness, const char *attr_name, int32_t attr_dim,
                      float *attr_out, const char *model_params, int64_t bmesh_nv,
                      const float *bmesh_x, const float *bmesh_v, int64_t bmesh_nt,
                      const int32_t *bmesh_tris, const char *bgrid_type, int64_t tracker_nq,
                      const int32_t *tracker_quads) {
  using namespace zeno;
  try {
    Graph g;
    auto num = [](float v) { return std::make_shared<NumericObject>(v); };
    auto inum = [](int v) { return std::make_shared<NumericObject>(v); };
    auto str = [](const char *v) { return std::make_shared<StringObject>(v); };
    auto prim = std::make_shared<PrimitiveObject>();
    auto &p = prim->verts();
    auto &pv = prim->attrs3["vel"];
    p.resize(n);
    pv.resize(n);
    for (int64_t i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
        p[i][d] = pos[3 * i + d];
        pv[i][d] = vel ? vel[3 * i + d] : 0.0f;
      }

    g.addNode("ConfigConstitutiveModel", "model");
    g.setNodeInput("model", "dx", num(dx));
    g.setNodeInput("model", "ppc", num(ppc));
    g.setNodeInput("model", "density", num(density));
    g.setNodeInput("model", "type", str(type));
    g.setNodeInput("model", "plasticity", str(plasticity));
    g.setNodeInput("model", "E", num(E));
    g.setNodeInput("model", "nu", num(nu));
    // ConfigConstitutiveModel "params": "key=value;key=value" as a DictObject
    // of NumericObjects, the way a zeno graph feeds that socket
    if (model_params && model_params[0]) {
      auto dict = std::make_shared<DictObject>();
      std::istringstream ps(model_params);
      std::string item;
      while (std::getline(ps, item, ';')) {
        const size_t eq = item.find('=');
        if (eq == std::string::npos) continue;
        dict->lut[item.substr(0, eq)] = num(std::stof(item.substr(eq + 1)));
      }
      g.setNodeInput("model", "params", dict);
    }
    g.addNode("ToZSParticles", "pars");
    g.bindNodeInput("pars", "ZSModel", "model", "ZSModel");
    g.setNodeInput("pars", "prim", prim);
    g.addNode("MakeZSPartition", "table");
    g.addNode("MakeZSGrid", "grid");
    g.setNodeInput("grid", "dx", num(dx));
    g.setNodeInput("grid", "transfer", str(transfer ? transfer : "apic"));
    g.addNode("ToZSBoundary", "bnd");
    g.setNodeInput("bnd", "type", str(bc_type));
    g.setNodeInput("bnd", "dx", num(dx));
    g.setNodeInput("bnd", "thickness", inum(bc_thickness));
    for (const char *id : {"model", "pars", "table", "grid", "bnd"}) g.markOnce(id);
    // optional level-set collider: ls = {dx, center[3], radius, height, extent,
    // translation[3], translation_rate[3], scale, scale_rate, ypr[3]}
    const bool collider = ls_shape && ls && std::string(ls_shape) != "none";
    if (collider) {
      auto v3 = [](const float *a) { return std::make_shared<NumericObject>(vec3f{a[0], a[1], a[2]}); };
      g.addNode("MakeZSLevelSet", "ls");
      g.setNodeInput("ls", "dx", num(ls[0]));
      g.setNodeInput("ls", "shape", str(ls_shape));
      g.setNodeInput("ls", "center", v3(ls + 1));
      g.setNodeInput("ls", "radius", num(ls[4]));
      g.setNodeInput("ls", "height", num(ls[5]));
      g.setNodeInput("ls", "extent", num(ls[6]));
      g.addNode("ToZSBoundary", "lsb");
      g.bindNodeInput("lsb", "ZSLevelSet", "ls", "ZSLevelSet");
      g.setNodeInput("lsb", "translation", v3(ls + 7));
      g.setNodeInput("lsb", "translation_rate", v3(ls + 10));
      g.setNodeInput("lsb", "scale", num(ls[13]));
      g.setNodeInput("lsb", "scale_rate", num(ls[14]));
      g.setNodeInput("lsb", "ypr_angles", v3(ls + 15));
      g.setNodeInput("lsb", "type", str(ls_type ? ls_type : "sticky"));
      g.markOnce("ls");
      g.markOnce("lsb");
    }
    // optional cloth: cloth_params = {stiffness_shear, stiffness_normal,
    // friction_angle, damping_coeff}; the same model as the particles
    std::shared_ptr<PrimitiveObject> cprim;
    const bool cloth = cloth_nv > 0 && cloth_x && cloth_nt > 0 && cloth_tris && cloth_params;
    if (cloth) {
      cprim = std::make_shared<PrimitiveObject>();
      auto &cp = cprim->verts();
      cp.resize(cloth_nv);
      auto &cv = cprim->attrs3["vel"];
      cv.resize(cloth_nv);
      for (int64_t i = 0; i < cloth_nv; ++i)
        for (int d = 0; d < 3; ++d) {
          cp[i][d] = cloth_x[3 * i + d];
          cv[i][d] = cloth_v ? cloth_v[3 * i + d] : 0.0f;
        }
      cprim->tris.resize(cloth_nt);
      for (int64_t i = 0; i < cloth_nt; ++i)
        for (int d = 0; d < 3; ++d) cprim->tris[i][d] = cloth_tris[3 * i + d];
      g.addNode("ToZSCloth", "cloth");
      g.bindNodeInput("cloth", "ZSModel", "model", "ZSModel");
      g.setNodeInput("cloth", "prim", cprim);
      g.setNodeInput("cloth", "stiffness_shear", num(cloth_params[0]));
      g.setNodeInput("cloth", "stiffness_normal", num(cloth_params[1]));
      g.setNodeInput("cloth", "friction_angle", num(cloth_params[2]));
      g.setNodeInput("cloth", "damping_coeff", num(cloth_params[3]));
      g.markOnce("cloth");
    }
    // optional ConstructBendingSprings on the cloth
    const bool bending = cloth && bending_type && bending_type[0];
    if (bending) {
      g.addNode("ConstructBendingSprings", "bend");
      g.bindNodeInput("bend", "ZSSurfPrim", "cloth", "ZSParticles");
      g.setNodeInput("bend", "bending_stiffness", num(bending_stiffness));
      g.setNodeInput("bend", "type:", str(bending_type));
      g.markOnce("bend");
    }
    // optional tracker points (ToTrackerParticles), moved by the grid
    std::shared_ptr<PrimitiveObject> tprim;
    const bool trackers = tracker_n > 0 && tracker_x;
    if (trackers) {
      tprim = std::make_shared<PrimitiveObject>();
      auto &tp = tprim->verts();
      tp.resize(tracker_n);
      for (int64_t i = 0; i < tracker_n; ++i)
        for (int d = 0; d < 3; ++d) tp[i][d] = tracker_x[3 * i + d];
      if (tracker_quads && tracker_nq > 0) {  // a tetrahedral mesh's vertices
        tprim->quads.resize(tracker_nq);
        for (int64_t i = 0; i < tracker_nq; ++i)
          for (int d = 0; d < 4; ++d) tprim->quads[i][d] = tracker_quads[4 * i + d];
        g.addNode("ToZSParticles", "trk");
        g.bindNodeInput("trk", "ZSModel", "model", "ZSModel");
        g.setNodeInput("trk", "category", inum(3));
      } else {
        g.addNode("ToTrackerParticles", "trk");
      }
      g.setNodeInput("trk", "prim", tprim);
      g.markOnce("trk");
    }
    // optional boundary grid: a triangle mesh through ToBoundaryParticles,
    // its own partition and grid of transfer "boundary" and
    // ZSBoundaryPrimitiveToZSGrid, applied with bgrid_type after the walls
    // (and the collider)
    std::shared_ptr<PrimitiveObject> bprim;
    const bool bgrid = bmesh_nv > 0 && bmesh_x && bmesh_nt > 0 && bmesh_tris && bgrid_type;
    if (bgrid) {
      bprim = std::make_shared<PrimitiveObject>();
      auto &bp = bprim->verts();
      bp.resize(bmesh_nv);
      auto &bv = bprim->attrs3["vel"];
      bv.resize(bmesh_nv);
      for (int64_t i = 0; i < bmesh_nv; ++i)
        for (int d = 0; d < 3; ++d) {
          bp[i][d] = bmesh_x[3 * i + d];
          bv[i][d] = bmesh_v ? bmesh_v[3 * i + d] : 0.0f;
        }
      bprim->tris.resize(bmesh_nt);
      for (int64_t i = 0; i < bmesh_nt; ++i)
        for (int d = 0; d < 3; ++d) bprim->tris[i][d] = bmesh_tris[3 * i + d];
      g.addNode("ToBoundaryParticles", "bpars");
      g.setNodeInput("bpars", "prim", bprim);
      g.setNodeInput("bpars", "dx", num(dx));
      g.addNode("MakeZSPartition", "btable");
      g.addNode("MakeZSGrid", "bgrid0");
      g.setNodeInput("bgrid0", "dx", num(dx));
      g.setNodeInput("bgrid0", "transfer", str("boundary"));
      g.addNode("ZSPartitionForZSParticles", "bpart");
      g.bindNodeInput("bpart", "ZSPartition", "btable", "ZSPartition");
      g.bindNodeInput("bpart", "ZSGrid", "bgrid0", "ZSGrid");
      g.bindNodeInput("bpart", "ZSParticles", "bpars", "ZSParticles");
      g.addNode("ZSGridFromZSPartition", "bclear");
      g.bindNodeInput("bclear", "ZSPartition", "bpart", "ZSPartition");
      g.bindNodeInput("bclear", "ZSGrid", "bgrid0", "ZSGrid");
      g.addNode("ZSBoundaryPrimitiveToZSGrid", "bp2g");
      g.bindNodeInput("bp2g", "ZSParticles", "bpars", "ZSParticles");
      g.bindNodeInput("bp2g", "ZSPartition", "bpart", "ZSPartition");
      g.bindNodeInput("bp2g", "ZSGrid", "bclear", "ZSGrid");
      g.addNode("UpdateZSGrid", "bupd");
      g.bindNodeInput("bupd", "ZSPartition", "bpart", "ZSPartition");
      g.bindNodeInput("bupd", "ZSGrid", "bp2g", "ZSGrid");
      g.setNodeInput("bupd", "dt", num(dt));
      for (const char *id : {"bpars", "btable", "bgrid0", "bpart", "bclear", "bp2g", "bupd"})
        g.markOnce(id);
    }
    auto dtobj = num(dt);
    std::string last;
    if (fused) {
      g.addNode("ZSMPMSubstep", "step");
      g.bindNodeInput("step", "ZSParticles", "pars", "ZSParticles");
      g.bindNodeInput("step", "ZSBoundary", "bnd", "ZSBoundary");
      if (collider) g.bindNodeInput("step", "ZSCollider", "lsb", "ZSBoundary");
      g.bindNodeInput("step", "ZSGrid", "grid", "ZSGrid");
      if (cloth) g.bindNodeInput("step", "ZSCloth", "cloth", "ZSParticles");
      if (trackers) g.bindNodeInput("step", "ZSTrackers", "trk", "ZSParticles");
      if (bending) g.bindNodeInput("step", "ZSBending", "bend", "ZSSpringPrim");
      if (bgrid) {
        g.bindNodeInput("step", "BoundaryZSGrid", "bupd", "ZSGrid");
        g.setNodeInput("step", "boundary_type", str(bgrid_type));
      }
      g.setNodeInput("step", "dt", dtobj);
      g.setNodeInput("step", "gravity", num(gravity));
      g.setNodeInput("step", "substeps", inum(substeps));
      g.applyNodes({"step"});
      last = "step";
    } else {
      g.addNode("ZSPartitionForZSParticles", "part");
      g.bindNodeInput("part", "ZSPartition", "table", "ZSPartition");
      g.bindNodeInput("part", "ZSGrid", "grid", "ZSGrid");
      g.bindNodeInput("part", "ZSParticles", "pars", "ZSParticles");
      if (cloth) g.bindNodeInput("part", "ZSCloth", "cloth", "ZSParticles");
      if (trackers) g.bindNodeInput("part", "ZSTrackers", "trk", "ZSParticles");
      if (bending) g.bindNodeInput("part", "ZSBending", "bend", "ZSSpringPrim");
      g.addNode("ExpandZSPartition", "expand");
      g.bindNodeInput("expand", "ZSPartition", "part", "ZSPartition");
      g.addNode("ZSGridFromZSPartition", "clear");
      g.bindNodeInput("clear", "ZSPartition", "expand", "ZSPartition");
      g.bindNodeInput("clear", "ZSGrid", "grid", "ZSGrid");
      g.addNode("ZSParticleToZSGrid", "p2g");
      g.bindNodeInput("p2g", "ZSParticles", "pars", "ZSParticles");
      g.bindNodeInput("p2g", "ZSPartition", "expand", "ZSPartition");
      g.bindNodeInput("p2g", "ZSGrid", "clear", "ZSGrid");
      g.setNodeInput("p2g", "dt", dtobj);
      g.addNode("UpdateZSGrid", "update");
      g.bindNodeInput("update", "ZSPartition", "expand", "ZSPartition");
      g.bindNodeInput("update", "ZSGrid", "p2g", "ZSGrid");
      g.setNodeInput("update", "dt", dtobj);
      g.setNodeInput("update", "gravity", num(gravity));
      g.addNode("ApplyBoundaryOnZSGrid", "bc");
      g.bindNodeInput("bc", "ZSPartition", "expand", "ZSPartition");
      g.bindNodeInput("bc", "ZSGrid", "update", "ZSGrid");
      g.bindNodeInput("bc", "ZSBoundary", "bnd", "ZSBoundary");
      const char *grid_src = "bc";
      if (collider) {
        // StepZSBoundary then the collider, after the walls, every substep
        g.addNode("StepZSBoundary", "stepb");
        g.bindNodeInput("stepb", "ZSBoundary", "lsb", "ZSBoundary");
        g.setNodeInput("stepb", "dt", dtobj);
        g.addNode("ApplyBoundaryOnZSGrid", "bc2");
        g.bindNodeInput("bc2", "ZSPartition", "expand", "ZSPartition");
        g.bindNodeInput("bc2", "ZSGrid", "bc", "ZSGrid");
        g.bindNodeInput("bc2", "ZSBoundary", "stepb", "ZSBoundary");
        grid_src = "bc2";
      }
      if (bgrid) {
        g.addNode("ApplyGridBoundaryOnZSGrid", "gbc");
        g.bindNodeInput("gbc", "ZSPartition", "expand", "ZSPartition");
        g.bindNodeInput("gbc", "ZSGrid", grid_src, "ZSGrid");
        g.bindNodeInput("gbc", "BoundaryZSPartition", "bpart", "ZSPartition");
        g.bindNodeInput("gbc", "BoundaryZSGrid", "bupd", "ZSGrid");
        g.setNodeInput("gbc", "type:", str(bgrid_type));
        grid_src = "gbc";
      }
      g.addNode("ZSGridToZSParticle", "g2p");
      g.bindNodeInput("g2p", "ZSGrid", grid_src, "ZSGrid");
      g.bindNodeInput("g2p", "ZSPartition", "expand", "ZSPartition");
      g.bindNodeInput("g2p", "ZSParticles", "pars", "ZSParticles");
      g.setNodeInput("g2p", "dt", dtobj);
      g.addNode("ZSReturnMapping", "rm");
      g.bindNodeInput("rm", "ZSParticles", "g2p", "ZSParticles");
      for (int32_t k = 0; k < substeps; ++k) g.applyNodes({"rm"});
      last = "rm";
      if (out_max_vel_sqr && substeps > 0)
        *out_max_vel_sqr =
            std::dynamic_pointer_cast<NumericObject>(g.getNodeOutput("update", "MaxVelSqr"))
                ->get<float>();
    }
    if (fused && out_max_vel_sqr)
      *out_max_vel_sqr =
          std::dynamic_pointer_cast<NumericObject>(g.getNodeOutput("step", "MaxVelSqr"))
              ->get<float>();
    g.addNode("UpdatePrimitiveFromZSParticles", "out");
    g.setNodeInput("out", "ZSParticles", g.getNodeOutput(last, "ZSParticles"));
    g.applyNodes({"out"});
    if (attr_name && attr_name[0] && attr_out) {  // UpdatePrimitiveAttrFromZSParticles
      g.addNode("UpdatePrimitiveAttrFromZSParticles", "attr");
      g.setNodeInput("attr", "ZSParticles", g.getNodeOutput(last, "ZSParticles"));
      g.setNodeInput("attr", "attr", str(attr_name));
      g.setNodeInput("attr", "type:", str(attr_dim == 1 ? "float" : "vec3f"));
      g.applyNodes({"attr"});
      const std::string key = std::string(attr_name) == "x" ? "pos" : attr_name;
      if (attr_dim == 1) {
        const auto &a = prim->attrs1.at(key);
        for (int64_t i = 0; i < n; ++i) attr_out[i] = a[i];
      } else {
        const auto &a = prim->attrs3.at(key);
        for (int64_t i = 0; i < n; ++i)
          for (int d = 0; d < 3; ++d) attr_out[3 * i + d] = a[i][d];
      }
    }
    if (write_path && write_path[0]) {  // ComputeVonMises -> WriteZSParticles
      g.addNode("ComputeVonMises", "vms");
      g.setNodeInput("vms", "ZSParticles", g.getNodeOutput(last, "ZSParticles"));
      g.addNode("WriteZSParticles", "write");
      g.bindNodeInput("write", "ZSParticles", "vms", "ZSParticles");
      g.setNodeInput("write", "path", str(write_path));
      g.applyNodes({"write"});
    }
    for (int64_t i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
        out_x[3 * i + d] = p[i][d];
        out_v[3 * i + d] = pv[i][d];
      }
    if (cloth) {  // UpdatePrimitiveFromZSParticles on the cloth
      g.addNode("UpdatePrimitiveFromZSParticles", "cout");
      g.setNodeInput("cout", "ZSParticles", g.getNodeOutput("cloth", "ZSParticles"));
      g.applyNodes({"cout"});
      const auto &cp = cprim->verts();
      const auto &cv = cprim->attrs3["vel"];
      for (int64_t i = 0; i < cloth_nv; ++i)
        for (int d = 0; d < 3; ++d) {
          if (cloth_out_x) cloth_out_x[3 * i + d] = cp[i][d];
          if (cloth_out_v) cloth_out_v[3 * i + d] = cv[i][d];
        }
    }
    if (trackers) {  // UpdatePrimitiveFromZSParticles on the trackers
      g.addNode("UpdatePrimitiveFromZSParticles", "tout");
      g.setNodeInput("tout", "ZSParticles", g.getNodeOutput("trk", "ZSParticles"));
      g.applyNodes({"tout"});
      const auto &tp = tprim->verts();
      const auto &tv = tprim->attrs3["vel"];
      for (int64_t i = 0; i < tracker_n; ++i)
        for (int d = 0; d < 3; ++d) {
          if (tracker_out_x) tracker_out_x[3 * i + d] = tp[i][d];
          if (tracker_out_v) tracker_out_v[3 * i + d] = tv[i][d];
        }
    }
    return 0;
  } catch (const std::exception &e) {
    copy_out(e.what(), err, err_cap);
    return 1;
  }
}

}  // extern "C"
