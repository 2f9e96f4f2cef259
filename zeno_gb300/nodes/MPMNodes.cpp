// The CuLagrange MPM nodes of zeno (projects/CuLagrange/mpm/*.cu) as thin
// wrappers over the zsmpm C ABI: same node names, socket names, parameter
// names and defaults, same in-place object flow (a node mutates its input
// object and emits the same pointer).  The zpc containers the reference
// passes between nodes become one device context per particle set, shared
// by the ZSParticles, ZSPartition and ZSGrid objects once they are bound.
#include <zsmpm.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#ifdef ZSMPM_WITH_ZENO
// inside zeno: the real node API (projects/CuLagrange/CMakeLists.txt adds
// this file to the zeno target)
#include <zeno/types/DictObject.h>
#include <zeno/types/NumericObject.h>
#include <zeno/types/PrimitiveObject.h>
#include <zeno/types/StringObject.h>
#include <zeno/zeno.h>
namespace zeno {
namespace prim_access {
inline std::vector<vec3f> &pos(PrimitiveObject &p) { return p.verts.values; }
inline std::vector<vec3f> *vel(PrimitiveObject &p, bool create) {
  if (!p.verts.has_attr("vel")) {
    if (!create) return nullptr;
    p.verts.add_attr<vec3f>("vel");
  }
  return &p.verts.attr<vec3f>("vel");
}
inline const std::vector<float> *float_attr(PrimitiveObject &p, const std::string &k) {
  return p.verts.has_attr(k) ? &p.verts.attr<float>(k) : nullptr;
}
inline const std::vector<vec3i> &tris(PrimitiveObject &p) { return p.tris.values; }
inline const std::vector<vec2i> &lines(PrimitiveObject &p) { return p.lines.values; }
inline const std::vector<vec4i> &quads(PrimitiveObject &p) { return p.quads.values; }
// float / vec3f attribute `k` of the vertices (tris: of the triangles),
// created when absent, sized to the element count
template <class T> std::vector<T> &attr(PrimitiveObject &p, bool tris, const std::string &k) {
  if (tris) {
    if (!p.tris.has_attr(k)) p.tris.add_attr<T>(k);
    return p.tris.attr<T>(k);
  }
  if (!p.verts.has_attr(k)) p.verts.add_attr<T>(k);
  return p.verts.attr<T>(k);
}
}  // namespace prim_access
}  // namespace zeno
#else
// headless: the mirror of the node API
#include "zeno_api.hpp"
namespace zeno {
namespace prim_access {
inline std::vector<vec3f> &pos(PrimitiveObject &p) { return p.verts(); }
inline std::vector<vec3f> *vel(PrimitiveObject &p, bool create) {
  auto it = p.attrs3.find("vel");
  if (it == p.attrs3.end()) {
    if (!create) return nullptr;
    return &p.attrs3["vel"];
  }
  return &it->second;
}
inline const std::vector<float> *float_attr(PrimitiveObject &p, const std::string &k) {
  auto it = p.attrs1.find(k);
  return it == p.attrs1.end() ? nullptr : &it->second;
}
inline const std::vector<vec3i> &tris(PrimitiveObject &p) { return p.tris; }
inline const std::vector<vec2i> &lines(PrimitiveObject &p) { return p.lines; }
inline const std::vector<vec4i> &quads(PrimitiveObject &p) { return p.quads; }
template <class T> std::vector<T> &attr(PrimitiveObject &p, bool tris, const std::string &k) {
  const size_t n = tris ? p.tris.size() : p.size();
  std::vector<T> *a;
  if constexpr (std::is_same_v<T, float>)
    a = tris ? &p.tri_attrs1[k] : &p.attrs1[k];
  else
    a = tris ? &p.tri_attrs3[k] : (k == "pos" ? &p.verts() : &p.attrs3[k]);
  a->resize(n);
  return *a;
}
}  // namespace prim_access
}  // namespace zeno
#endif

namespace zeno {

namespace {

void check(int32_t rc, const char *what) {
  if (rc != MPM_OK)
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(rc) +
                             "): " + mpm_last_error());
}

}  // namespace

// One device context: grid + partition + particle store of a particle set.
struct MpmContext {
  mpm_ctx *h = nullptr;
  float dx = 0.0f;
  // the boundary points (a ToBoundaryParticles object) and type of the
  // boundary grid set in this context
  const void *bnd_src = nullptr;
  int32_t bnd_type = 0;
  ~MpmContext() {
    if (h) mpm_ctx_destroy(h);
  }
};

// ConfigConstitutiveModel output (Structures.hpp:34-132)
struct ZenoConstitutiveModel : IObject {
  mpm_material mat{};
  float dx = 0.1f, volume = 0.0f, density = 1000.0f;
};

// The material and particle volume a ZSModel object carries (false: the
// object is not a ZSModel); lets a host inspect what ConfigConstitutiveModel
// made of its inputs.
bool zsmodel_material(const zany &obj, mpm_material *mat, float *volume) {
  auto m = std::dynamic_pointer_cast<ZenoConstitutiveModel>(obj);
  if (!m) return false;
  if (mat) *mat = m->mat;
  if (volume) *volume = m->volume;
  return true;
}

// ToZSParticles output (Structures.hpp:134-531)
struct ZenoParticles : IObject {
  std::shared_ptr<MpmContext> ctx;
  // ToZSCloth: the mesh and cloth parameters, attached to the context of the
  // particles it is stepped with (one cloth per context)
  bool cloth = false;
  mpm_cloth_desc cloth_desc{};
  std::weak_ptr<MpmContext> cloth_ctx;
  // ToTrackerParticles: massless points carried by the grid velocity,
  // attached to the context of the particles they are stepped with
  bool tracker = false;
  std::weak_ptr<MpmContext> tracker_ctx;
  // ConstructBendingSprings: springs over the vertices of the ToZSCloth cloth
  // `surf`, added to the context that steps that cloth
  bool bending = false;
  int32_t bending_type = MPM_BENDING_VERTEX;
  float bending_stiffness = 0.0f;
  std::shared_ptr<ZenoParticles> surf;
  std::weak_ptr<MpmContext> bending_ctx;
  std::shared_ptr<PrimitiveObject> prim;  // the source primitive, written back by
                                          // UpdatePrimitiveFromZSParticles
  std::shared_ptr<ZenoConstitutiveModel> model;
  int64_t n = 0;
  int category = 0;
  // ToBoundaryParticles: points of a boundary mesh (the vertices, then one
  // per triangle) for a boundary grid, kept on the host
  bool boundary = false;
  float bdx = 0.0f;
  int64_t b_verts = 0, b_n = 0;
  std::vector<float> bx, bv, bm, bnrm;
};

// MakeZSPartition output (Structures.hpp:533-586)
struct ZenoPartition : IObject {
  std::shared_ptr<MpmContext> ctx;
  bool rebuilt = false;
  std::shared_ptr<ZenoParticles> bnd;  // the partition of boundary points
};

// MakeZSGrid output (Structures.hpp:588-623)
struct ZenoGrid : IObject {
  float dx = 0.1f;
  std::string transferScheme = "apic";
  std::shared_ptr<MpmContext> ctx;
  std::shared_ptr<ZenoPartition> partition;
  std::shared_ptr<ZenoParticles> bnd;  // transfer "boundary": the points it holds
};

// MakeZSLevelSet output (Structures.hpp: ZenoLevelSet): here a dense grid of
// signed distances (x fastest) at origin + (i, j, k) * dx, with an optional
// material velocity field (3 planes) or a constant velocity
struct ZenoLevelSet : IObject {
  float dx = 0.1f;
  std::string transferScheme = "unknown", category = "cellcentered";
  int dims[3] = {0, 0, 0};
  vec3f origin{0.f, 0.f, 0.f};
  std::vector<float> sdf;
  std::vector<float> vel;  // empty or 3 * dims product
  vec3f const_vel{0.f, 0.f, 0.f};
};

// ToZSBoundary output (Structures.hpp:807-835): the analytic box walls, or a
// level-set collider with its transform (attached to a context on first use)
struct ZenoBoundary : IObject {
  mpm_boundary bc{};
  std::shared_ptr<ZenoLevelSet> ls;
  mpm_collider_desc col{};
  std::weak_ptr<MpmContext> attached;
  int32_t collider_id = -1;
};

namespace {

float get_dt(const INode &node) {
  return node.get_input<NumericObject>("dt")->get<float>();
}

// Make a boundary take effect in the context: box walls replace the
// context's walls; a level-set collider joins the context's colliders once
// (every boundary application then resolves the walls and all colliders,
// each projection being idempotent).
void attach_boundary(const std::shared_ptr<MpmContext> &ctx, ZenoBoundary &b) {
  if (!b.ls) {
    check(mpm_set_boundary(ctx->h, &b.bc), "mpm_set_boundary");
    return;
  }
  if (b.attached.lock() == ctx) return;
  mpm_collider_desc c = b.col;
  const ZenoLevelSet &ls = *b.ls;
  for (int a = 0; a < 3; ++a) {
    c.dims[a] = ls.dims[a];
    c.origin[a] = ls.origin[a];
    c.const_velocity[a] = ls.const_vel[a];
  }
  c.spacing = ls.dx;
  c.sdf = ls.sdf.data();
  c.velocity = ls.vel.empty() ? nullptr : ls.vel.data();
  int32_t id = -1;
  check(mpm_add_collider(ctx->h, &c, &id), "mpm_add_collider");
  b.attached = ctx;
  b.collider_id = id;
}

// MakeZSGrid "transfer" -> MPM_TRANSFER_*
int32_t transfer_of(const ZenoGrid &g) {
  if (g.transferScheme == "flip") return MPM_TRANSFER_FLIP;
  if (g.transferScheme == "aflip") return MPM_TRANSFER_AFLIP;
  return MPM_TRANSFER_APIC;
}

// A device context for a particle set / mesh on the current CUDA device: the
// directory covers [lo, hi] (the optional domain inputs), else the bounding
// box of `pos` plus 8 cells on every side, and grows (recentred on the
// particles) whenever one leaves it, as the reference's hashed block table
// takes new blocks (Structures.hpp:535).
std::shared_ptr<MpmContext> make_context(const ZenoConstitutiveModel &model,
                                         const std::vector<vec3f> &pos, const float *lo_in,
                                         const float *hi_in, int64_t max_particles) {
  const float dx = model.dx;
  float lo[3], hi[3];
  if (lo_in && hi_in) {
    for (int d = 0; d < 3; ++d) {
      lo[d] = lo_in[d];
      hi[d] = hi_in[d];
    }
  } else {
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::numeric_limits<float>::max();
      hi[d] = -std::numeric_limits<float>::max();
    }
    for (const auto &p : pos)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], p[d]);
        hi[d] = std::max(hi[d], p[d]);
      }
    if (pos.empty())
      for (int d = 0; d < 3; ++d) lo[d] = hi[d] = 0.0f;
    for (int d = 0; d < 3; ++d) {
      lo[d] -= 8.0f * dx;
      hi[d] += 8.0f * dx;
    }
  }
  mpm_ctx_desc desc{};
  desc.device = -1;  // the calling thread's current CUDA device
  desc.dx = dx;
  for (int d = 0; d < 3; ++d) {
    const int b0 = (int)std::floor(lo[d] / dx / 4.0f) - 1;
    const int b1 = (int)std::floor(hi[d] / dx / 4.0f) + 2;
    desc.block_lo[d] = b0;
    desc.block_dims[d] = std::max(3, b1 - b0 + 1);
  }
  desc.max_particles = std::max<int64_t>(max_particles, 1);
  auto ctx = std::make_shared<MpmContext>();
  ctx->dx = dx;
  check(mpm_ctx_create(&desc, &ctx->h), "mpm_ctx_create");
  check(mpm_set_materials(ctx->h, &model.mat, 1), "mpm_set_materials");
  check(mpm_set_auto_regrow(ctx->h, 1), "mpm_set_auto_regrow");
  return ctx;
}

// a ToZSCloth cloth joins the particles' context once; its primitive
// provides the mesh
void attach_cloth(const std::shared_ptr<MpmContext> &ctx, ZenoParticles &cl) {
  if (!cl.cloth) throw std::runtime_error("ZSCloth: the input is not a ToZSCloth output");
  if (cl.cloth_ctx.lock() == ctx) return;
  if (cl.cloth_ctx.lock()) throw std::runtime_error("ZSCloth: the cloth belongs to another context");
  auto &pos = prim_access::pos(*cl.prim);
  mpm_cloth_desc d = cl.cloth_desc;
  std::vector<int32_t> idx;
  if (d.kind == MPM_MESH_CURVE) {
    const auto &ln = prim_access::lines(*cl.prim);
    for (const auto &l : ln) idx.insert(idx.end(), {l[0], l[1]});
    d.n_tris = (int64_t)ln.size();
  } else {
    const auto &tr = prim_access::tris(*cl.prim);
    for (const auto &t : tr) idx.insert(idx.end(), {t[0], t[1], t[2]});
    d.n_tris = (int64_t)tr.size();
  }
  const auto *v = prim_access::vel(*cl.prim, false);
  d.n_verts = (int64_t)pos.size();
  d.x = pos.empty() ? nullptr : pos[0].data();
  d.v = v && v->size() == pos.size() ? (*v)[0].data() : nullptr;
  d.tris = idx.data();
  check(mpm_cloth_create(ctx->h, &d), "mpm_cloth_create");
  cl.cloth_ctx = ctx;
  cl.ctx = ctx;
}

// ToTrackerParticles points join the particles' context once; the
// primitive's "pos" ("vel" when present) seeds them
void attach_trackers(const std::shared_ptr<MpmContext> &ctx, ZenoParticles &tk) {
  if (!tk.tracker)
    throw std::runtime_error("ZSTrackers: the input is not a ToTrackerParticles output or a "
                             "tetrahedral ToZSParticles mesh");
  if (tk.tracker_ctx.lock() == ctx) return;
  if (tk.tracker_ctx.lock())
    throw std::runtime_error("ZSTrackers: the trackers belong to another context");
  auto &pos = prim_access::pos(*tk.prim);
  if (pos.empty()) throw std::runtime_error("ZSTrackers: the primitive has no points");
  const auto *v = prim_access::vel(*tk.prim, false);
  check(mpm_trackers_create(ctx->h, (int64_t)pos.size(), pos[0].data(),
                            v && v->size() == pos.size() ? (*v)[0].data() : nullptr),
        "mpm_trackers_create");
  tk.tracker_ctx = ctx;
  tk.ctx = ctx;
}

// ConstructBendingSprings springs join the context of their cloth once
void attach_bending(const std::shared_ptr<MpmContext> &ctx, ZenoParticles &bs) {
  if (!bs.bending || !bs.surf)
    throw std::runtime_error("ZSBending: the input is not a ConstructBendingSprings output");
  if (bs.bending_ctx.lock() == ctx) return;
  if (bs.bending_ctx.lock())
    throw std::runtime_error("ZSBending: the springs belong to another context");
  if (bs.surf->cloth_ctx.lock() != ctx)
    throw std::runtime_error("ZSBending: the springs' cloth is not stepped with these particles "
                             "(pass it as ZSCloth too)");
  const float thickness = bs.surf->model ? bs.surf->model->dx : ctx->dx;
  int64_t n = 0;
  check(mpm_cloth_add_bending(ctx->h, bs.bending_type, bs.bending_stiffness, thickness, &n),
        "mpm_cloth_add_bending");
  bs.bending_ctx = ctx;
  bs.n = n;
}

// a ToZSCloth cloth used on its own as the ZSParticles of a substep gets a
// context of its own (no particles)
void ensure_cloth_ctx(ZenoParticles &pars) {
  if (pars.tracker && !pars.ctx)
    throw std::runtime_error("tracker particles carry no mass: step them through the ZSTrackers "
                             "input with the particles that move them");
  if (pars.bending && !pars.ctx)
    throw std::runtime_error("bending springs are stepped through the ZSBending input, with "
                             "their cloth as ZSCloth");
  if (!pars.cloth || pars.ctx) return;
  auto ctx = make_context(*pars.model, prim_access::pos(*pars.prim), nullptr, nullptr, 1);
  check(mpm_particles_upload(ctx->h, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                             nullptr, nullptr, nullptr, nullptr),
        "mpm_particles_upload");
  attach_cloth(ctx, pars);
}

std::shared_ptr<MpmContext> bound_ctx(const std::shared_ptr<ZenoPartition> &p, const char *node) {
  if (!p->ctx)
    throw std::runtime_error(std::string(node) +
                             ": the ZSPartition is not bound to particles "
                             "(run ZSPartitionForZSParticles first)");
  return p->ctx;
}

}  // namespace

/// ConfigConstitutiveModel (Generation.cu:18-88)
struct ConfigConstitutiveModel : INode {
  void apply() override {
    auto out = std::make_shared<ZenoConstitutiveModel>();
    const float dx = get_input2<float>("dx");
    out->dx = dx;
    out->volume = dx * dx * dx / get_input2<float>("ppc");
    out->density = get_input2<float>("density");
    mpm_material &m = out->mat;
    m.E = get_input2<float>("E");
    m.nu = get_input2<float>("nu");
    m.density = out->density;
    // the "params" dict (Generation.cu:32,53-58): optional numbers by key,
    // read where the reference reads them; the equation-of-state fluid (an
    // extension of this backend) takes its bulk modulus and exponent there too
    auto params = has_input("params") ? get_input<DictObject>("params") : std::make_shared<DictObject>();
    auto get_arg = [&params](const char *tag, float defl) {
      auto it = params->lut.find(tag);
      if (it == params->lut.end()) return defl;
      auto num = std::dynamic_pointer_cast<NumericObject>(it->second);
      if (!num)
        throw std::runtime_error(std::string("ConfigConstitutiveModel: params[\"") + tag +
                                 "\"] is not a number");
      return num->get<float>();
    };
    m.friction_angle_deg = 35.0f;  // reference default (Generation.cu:70)
    m.bulk = get_arg("bulk", 1e4f);
    m.gamma = get_arg("gamma", 7.0f);
    m.yield_stress = 1e5f;
    m.cc_beta = 2.0f;
    m.cc_xi = 1.0f;
    const std::string type = get_input2<std::string>("type");
    if (type == "fcr")
      m.type = MPM_FCR;
    else if (type == "nhk")
      m.type = MPM_NHK;
    else if (type == "stvk")
      m.type = MPM_STVK;
    else if (type == "snhk")
      m.type = MPM_SNHK;
    else if (type == "eos")
      m.type = MPM_EOS;
    else
      throw std::runtime_error("unrecognized (isotropic) elastic model [" + type + "]");
    if (get_input2<std::string>("aniso") != "none")
      throw std::runtime_error("anisotropic models are not supported by this MPM backend");
    // plasticity runs on StvkWithHencky (Generation.cu:66-82), with its
    // parameters from "params" and the reference's defaults
    const std::string plastic = get_input2<std::string>("plasticity");
    if (plastic == "nadp") {
      m.type = MPM_STVK;
      m.plasticity = MPM_PLASTIC_NADP;
      m.friction_angle_deg = get_arg("friction_angle", 35.0f);  // Generation.cu:69-70
    } else if (plastic == "navm") {
      m.type = MPM_STVK;
      m.plasticity = MPM_PLASTIC_NAVM;
      m.yield_stress = get_arg("yield_stress", 1e5f);  // Generation.cu:73-75
    } else if (plastic == "nacc") {
      m.type = MPM_STVK;
      m.plasticity = MPM_PLASTIC_NACC;
      m.friction_angle_deg = get_arg("friction_angle", 35.0f);  // Generation.cu:77-82
      m.cc_beta = get_arg("beta", 2.0f);
      m.cc_xi = get_arg("xi", 1.0f);
    } else if (plastic == "none") {
      m.plasticity = MPM_PLASTIC_NONE;
    } else {
      throw std::runtime_error("plasticity [" + plastic + "] is not supported by this MPM backend");
    }
    set_output("ZSModel", out);
  }
};
ZENDEFNODE(ConfigConstitutiveModel, {
                                        {{"float", "dx", "0.1"},
                                         {"float", "ppc", "8"},
                                         {"float", "density", "1000"},
                                         {"enum fcr nhk stvk snhk eos", "type", "fcr"},
                                         {"enum none arap", "aniso", "none"},
                                         {"enum none nadp navm nacc", "plasticity", "none"},
                                         {"float", "E", "10000"},
                                         {"float", "nu", "0.4"},
                                         {"DictObject:NumericObject", "params"}},
                                        {"ZSModel"},
                                        {},
                                        {"MPM"},
                                    });

/// ToZSCloth (Generation.cpp:432-689): a triangle mesh as codimensional
/// cloth with the model's in-plane elasticity; the cloth joins the context of
/// the particles it is stepped with (ZSMPMSubstep / ZSPartitionForZSParticles
/// input "ZSCloth").
struct ToZSCloth : INode {
  void apply() override {
    auto model = get_input<ZenoConstitutiveModel>("ZSModel");
    auto prim = get_input<PrimitiveObject>("prim");
    if (prim_access::tris(*prim).empty())
      throw std::runtime_error("ToZSCloth: the primitive has no triangles");
    const int type = model->mat.type;
    if (type != MPM_FCR && type != MPM_NHK && type != MPM_STVK)
      throw std::runtime_error("ToZSCloth: the model must be fcr, nhk or stvk");
    auto out = std::make_shared<ZenoParticles>();
    out->prim = prim;
    out->model = model;
    out->cloth = true;
    out->category = 2;  // ZenoParticles::surface
    mpm_cloth_desc &d = out->cloth_desc;
    d.model = type;
    d.E = model->mat.E;
    d.nu = model->mat.nu;
    d.density = model->density;
    d.stiffness_shear = get_input2<float>("stiffness_shear");
    d.stiffness_normal = get_input2<float>("stiffness_normal");
    d.friction_angle = get_input2<float>("friction_angle");
    d.damping_coeff = get_input2<float>("damping_coeff");
    set_output("ZSParticles", out);
  }
};
ZENDEFNODE(ToZSCloth, {
                          {"ZSModel",
                           "prim",
                           {"float", "stiffness_shear", "0."},
                           {"float", "stiffness_normal", "800."},
                           {"float", "friction_angle", "0."},
                           {"float", "damping_coeff", "0."}},
                          {"ZSParticles"},
                          {},
                          {"MPM"},
                      });

/// ConstructBendingSprings (Generation.cu:563-1001) on a ToZSCloth cloth:
/// "vertex" springs between the vertices opposite each interior edge (k =
/// E / (24 (1 - nu^2)) bending_stiffness, rest length at attachment), pushing
/// them apart while compressed; "angle" hinges, whose force is identically
/// zero in the reference (Transfer.cu:466-480); "element" (the reference's
/// default) is undefined there (its pairs are tagged as vertex springs
/// without vertex indices) and fails when attached.  The springs join the
/// substep through the ZSBending input of ZSPartitionForZSParticles or
/// ZSMPMSubstep, with their cloth as ZSCloth.
struct ConstructBendingSprings : INode {
  void apply() override {
    auto surf = get_input<ZenoParticles>("ZSSurfPrim");
    if (!surf->cloth || surf->cloth_desc.kind != MPM_MESH_SURFACE)
      throw std::runtime_error("ConstructBendingSprings: ZSSurfPrim is not a ToZSCloth surface");
    const std::string type = get_param<std::string>("type");
    auto out = std::make_shared<ZenoParticles>();
    out->bending = true;
    if (type == "vertex")
      out->bending_type = MPM_BENDING_VERTEX;
    else if (type == "element")
      out->bending_type = MPM_BENDING_ELEMENT;
    else if (type == "angle")
      out->bending_type = MPM_BENDING_ANGLE;
    else
      throw std::runtime_error("ConstructBendingSprings: unknown type [" + type + "]");
    out->bending_stiffness = get_input2<float>("bending_stiffness");
    out->surf = surf;
    out->model = surf->model;
    out->category = out->bending_type == MPM_BENDING_ANGLE ? 7 : 5;  // bending / vert_bending_spring
    set_output("ZSSpringPrim", out);
  }
};
ZENDEFNODE(ConstructBendingSprings, {
                                        {"ZSSurfPrim", {"float", "bending_stiffness", "0.01"}},
                                        {"ZSSpringPrim"},
                                        {{"enum vertex element angle", "type", "element"}},
                                        {"MPM"},
                                    });

/// ToTrackerParticles (Generation.cu:105-187): the primitive's points as
/// massless tracker particles that the substeps move with the grid's
/// velocity (v = sum W v_i, x += v dt; Transfer.cu:1259-1285).  They are
/// stepped with the particles of a ZSPartitionForZSParticles or ZSMPMSubstep
/// (input "ZSTrackers") and written back by UpdatePrimitiveFromZSParticles.
/// The reference's element centroids of a triangle primitive only feed its
/// wind impulse and are not kept.
struct ToTrackerParticles : INode {
  void apply() override {
    auto prim = get_input<PrimitiveObject>("prim");
    auto out = std::make_shared<ZenoParticles>();
    out->prim = prim;
    out->tracker = true;
    out->category = 4;  // ZenoParticles::tracker
    out->n = (int64_t)prim_access::pos(*prim).size();
    set_output("ZSParticles", out);
  }
};
ZENDEFNODE(ToTrackerParticles, {
                                   {"prim"},
                                   {"ZSParticles"},
                                   {},
                                   {"MPM"},
                               });

/// ToZSParticles (Generation.cpp:690-1145): m = vol * density, F = I, C = 0.
/// The device context is sized for the primitive: its block directory spans
/// the optional domain_min / domain_max inputs, else the bounding box plus 8
/// cells on every side, and grows whenever a particle leaves it.
struct ToZSParticles : INode {
  void apply() override {
    auto model = get_input<ZenoConstitutiveModel>("ZSModel");
    auto prim = get_input<PrimitiveObject>("prim");
    const auto &pos = prim_access::pos(*prim);
    const int64_t n = (int64_t)pos.size();
    auto out = std::make_shared<ZenoParticles>();
    out->prim = prim;
    out->model = model;
    out->n = n;
    out->category = get_input2<int>("category");
    float lo[3], hi[3];
    const bool domain = has_input<NumericObject>("domain_min") && has_input<NumericObject>("domain_max");
    if (domain) {
      auto a = get_input<NumericObject>("domain_min")->get<vec3f>();
      auto b = get_input<NumericObject>("domain_max")->get<vec3f>();
      for (int d = 0; d < 3; ++d) {
        lo[d] = a[d];
        hi[d] = b[d];
      }
    }
    if (out->category != 0 && !prim_access::quads(*prim).empty()) {
      // a tetrahedral mesh (Generation.cpp:740-741, 780-797): the reference's
      // transfers scatter nothing of it (ZSParticleToZSGrid takes surfaces and
      // curves only, Transfer.cu:1016-1036) and move its vertices with the
      // grid velocity (Transfer.cu:1287-1372); here its vertices are tracker
      // points, stepped through the ZSTrackers input of the particles whose
      // grid moves them
      out->tracker = true;
      out->category = 3;  // ZenoParticles::tet
      out->n = n;
      set_output("ZSParticles", out);
      return;
    }
    if (out->category != 0) {
      // a mesh (Generation.cpp:738-749): triangles become a surface (cloth),
      // segments a curve (hair), with the defaults of Generation.cpp:695-699
      // (k = 800, gamma = fa = dc = 0)
      const bool tri = !prim_access::tris(*prim).empty(), seg = !prim_access::lines(*prim).empty();
      if (!tri && !seg)
        throw std::runtime_error("ToZSParticles: category " + std::to_string(out->category) +
                                 " needs a tetrahedron, triangle or segment mesh");
      const int type = model->mat.type;
      if (type != MPM_FCR && type != MPM_NHK && type != MPM_STVK)
        throw std::runtime_error("ToZSParticles: a surface takes fcr, nhk or stvk");
      out->n = 0;
      out->cloth = true;
      out->category = tri ? 2 : 1;  // ZenoParticles::surface / curve
      mpm_cloth_desc &cd = out->cloth_desc;
      cd.kind = tri ? MPM_MESH_SURFACE : MPM_MESH_CURVE;
      cd.model = type;
      cd.E = model->mat.E;
      cd.nu = model->mat.nu;
      cd.density = model->density;
      cd.stiffness_shear = 0.0f;
      cd.stiffness_normal = 800.0f;
      cd.friction_angle = 0.0f;
      cd.damping_coeff = 0.0f;
      auto ctx = make_context(*model, pos, domain ? lo : nullptr, domain ? hi : nullptr, 1);
      check(mpm_particles_upload(ctx->h, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                 nullptr, nullptr, nullptr, nullptr),
            "mpm_particles_upload");
      attach_cloth(ctx, *out);
      set_output("ZSParticles", out);
      return;
    }
    auto ctx = make_context(*model, pos, domain ? lo : nullptr, domain ? hi : nullptr, n);
    std::vector<float> x(3 * n), v(3 * n, 0.0f), m(n, model->volume * model->density),
        vol(n, model->volume);
    for (int64_t i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) x[3 * i + d] = pos[i][d];
    if (auto *vel = prim_access::vel(*prim, false); vel && (int64_t)vel->size() == n)
      for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) v[3 * i + d] = (*vel)[i][d];
    // Cam-Clay particles start hardened at log(Jp) = -0.04, carried in the J
    // channel (Generation.cpp:987)
    std::vector<float> J;
    if (model->mat.plasticity == MPM_PLASTIC_NACC) J.assign(n, -0.04f);
    check(mpm_particles_upload(ctx->h, n, x.data(), v.data(), nullptr, nullptr,
                               J.empty() ? nullptr : J.data(), m.data(), vol.data(), nullptr,
                               nullptr, nullptr),
          "mpm_particles_upload");
    out->ctx = ctx;
    set_output("ZSParticles", out);
  }
};
ZENDEFNODE(ToZSParticles, {
                              {"ZSModel", "prim", {"int", "category", "0"}},
                              {"ZSParticles"},
                              {},
                              {"MPM"},
                          });

/// MakeZSPartition (Generation.cu:1470-1477)
struct MakeZSPartition : INode {
  void apply() override { set_output("ZSPartition", std::make_shared<ZenoPartition>()); }
};
ZENDEFNODE(MakeZSPartition, {
                                {},
                                {"ZSPartition"},
                                {},
                                {"MPM"},
                            });

/// MakeZSGrid (Generation.cu:1486-1512)
struct MakeZSGrid : INode {
  void apply() override {
    auto grid = std::make_shared<ZenoGrid>();
    grid->dx = get_input2<float>("dx");
    grid->transferScheme = get_input2<std::string>("transfer");
    const std::string &ts = grid->transferScheme;
    if (ts != "apic" && ts != "flip" && ts != "aflip" && ts != "boundary")
      throw std::runtime_error("unrecognized transfer scheme [" + ts + "]");
    set_output("ZSGrid", grid);
  }
};
ZENDEFNODE(MakeZSGrid, {
                           {{"float", "dx", "0.1"}, {"string", "transfer", "apic"}},
                           {"ZSGrid"},
                           {},
                           {"MPM"},
                       });

/// ZSPartitionForZSParticles (MPMPipeline.cu:21-112): bins the particles into
/// 4^3 blocks with the 1-ring halo and sorts them by (block, cell).  Both
/// strategies rebuild: a rebuild costs a few microseconds here.
struct ZSPartitionForZSParticles : INode {
  void apply() override {
    auto table = get_input<ZenoPartition>("ZSPartition");
    auto grid = get_input<ZenoGrid>("ZSGrid");
    auto pars = get_input<ZenoParticles>("ZSParticles");
    if (pars->boundary) {  // boundary points: their grid is built where it is applied
      if (grid->transferScheme != "boundary")
        throw std::runtime_error("boundary particles partition a grid of transfer [boundary]");
      table->bnd = pars;
      grid->bnd = pars;
      table->rebuilt = true;
      set_output("ZSPartition", table);
      return;
    }
    ensure_cloth_ctx(*pars);
    const std::string strategy = get_param<std::string>("strategy");
    if (strategy != "force" && strategy != "cache")
      throw std::runtime_error("unknown partition strategy [" + strategy + "]");
    if (std::fabs(grid->dx - pars->ctx->dx) > 1e-6f * pars->ctx->dx)
      throw std::runtime_error("ZSGrid dx differs from the dx of the particles' model");
    table->ctx = pars->ctx;
    grid->ctx = pars->ctx;
    check(mpm_set_transfer(pars->ctx->h, transfer_of(*grid)), "mpm_set_transfer");
    if (has_input<ZenoParticles>("ZSCloth"))  // a cloth stepped with these particles
      attach_cloth(pars->ctx, *get_input<ZenoParticles>("ZSCloth"));
    if (has_input<ZenoParticles>("ZSTrackers"))
      attach_trackers(pars->ctx, *get_input<ZenoParticles>("ZSTrackers"));
    if (has_input<ZenoParticles>("ZSBending"))
      attach_bending(pars->ctx, *get_input<ZenoParticles>("ZSBending"));
    check(mpm_partition(pars->ctx->h), "mpm_partition");
    table->rebuilt = true;
    set_output("ZSPartition", table);
  }
};
ZENDEFNODE(ZSPartitionForZSParticles, {
                                          {"ZSPartition", "ZSGrid", "ZSParticles", {"float", "ppb", "1"},
                                           "ZSCloth", "ZSTrackers", "ZSBending"},
                                          {"ZSPartition"},
                                          {{"enum force cache", "strategy", "force"}},
                                          {"MPM"},
                                      });

/// ExpandZSPartition (MPMPipeline.cu:121-231): the partition already holds
/// the 1-ring of neighbour blocks every quadratic stencil needs, so this node
/// only validates its parameters and passes the partition on.
struct ExpandZSPartition : INode {
  void apply() override {
    auto table = get_input<ZenoPartition>("ZSPartition");
    (void)get_param<int>("offset");
    (void)get_param<int>("extent");
    set_output("ZSPartition", table);
  }
};
ZENDEFNODE(ExpandZSPartition, {
                                  {"ZSPartition"},
                                  {"ZSPartition"},
                                  {{"int", "offset", "0"}, {"int", "extent", "2"}},
                                  {"MPM"},
                              });

/// ZSGridFromZSPartition (MPMPipeline.cu:241-267): size and clear the grid
struct ZSGridFromZSPartition : INode {
  void apply() override {
    auto table = get_input<ZenoPartition>("ZSPartition");
    auto grid = get_input<ZenoGrid>("ZSGrid");
    if (grid->transferScheme == "boundary") {  // cleared when its points are scattered
      grid->partition = table;
      set_output("ZSGrid", grid);
      return;
    }
    auto ctx = bound_ctx(table, "ZSGridFromZSPartition");
    grid->ctx = ctx;
    grid->partition = table;
    check(mpm_grid_clear(ctx->h), "mpm_grid_clear");
    set_output("ZSGrid", grid);
  }
};
ZENDEFNODE(ZSGridFromZSPartition, {
                                      {"ZSPartition", "ZSGrid"},
                                      {"ZSGrid"},
                                      {},
                                      {"MPM"},
                                  });

/// ZSParticleToZSGrid (Transfer.cu:985-1060), APIC transfer
struct ZSParticleToZSGrid : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    auto table = get_input<ZenoPartition>("ZSPartition");
    auto grid = get_input<ZenoGrid>("ZSGrid");
    auto ctx = bound_ctx(table, "ZSParticleToZSGrid");
    if (pars->ctx != ctx) throw std::runtime_error("ZSParticles and ZSPartition are not bound");
    check(mpm_p2g(ctx->h, get_dt(*this)), "mpm_p2g");
    set_output("ZSGrid", grid);
  }
};
ZENDEFNODE(ZSParticleToZSGrid, {
                                   {"ZSParticles", "ZSPartition", "ZSGrid", "dt"},
                                   {"ZSGrid"},
                                   {},
                                   {"MPM"},
                               });

/// UpdateZSGrid (MPMPipeline.cu:828-940): v = mv / m + accel dt, MaxVelSqr
struct UpdateZSGrid : INode {
  void apply() override {
    auto table = get_input<ZenoPartition>("ZSPartition");
    auto grid = get_input<ZenoGrid>("ZSGrid");
    if (grid->transferScheme == "boundary") {
      // v = mv / m and nrm = unit(nrm / m) (MPMPipeline.cu:899-911) are part
      // of building the boundary grid in the context that applies it
      set_output("ZSGrid", grid);
      set_output("MaxVelSqr", std::make_shared<NumericObject>(0.0f));
      return;
    }
    auto ctx = bound_ctx(table, "UpdateZSGrid");
    float acc[3] = {0.0f, get_input2<float>("gravity"), 0.0f};
    if (has_input("Accel")) {
      auto a = get_input<NumericObject>("Accel")->get<vec3f>();
      acc[0] = a[0];
      acc[1] = a[1];
      acc[2] = a[2];
    }
    check(mpm_set_gravity(ctx->h, acc[0], acc[1], acc[2]), "mpm_set_gravity");
    float vmax = 0.0f;
    check(mpm_grid_update(ctx->h, get_dt(*this), &vmax), "mpm_grid_update");
    set_output("ZSGrid", grid);
    set_output("MaxVelSqr", std::make_shared<NumericObject>(vmax));
  }
};
ZENDEFNODE(UpdateZSGrid, {
                             {{"float", "gravity", "-9.8"}, "ZSPartition", "ZSGrid", "dt", "Accel"},
                             {"ZSGrid", "MaxVelSqr"},
                             {},
                             {"MPM"},
                         });

/// MakeZSLevelSet (Generation.cu:1521-1595).  The reference makes an empty
/// sparse level set that VDB conversions fill; here the level set is a dense
/// grid of spacing dx, filled from `sdf_prim` (vertices on a regular grid of
/// `dims` samples, x fastest, float attribute "sdf", optional vec3
/// attribute "vel") or from an analytic `shape` (sphere of `radius` around
/// `center`; half-space y < `height` over `center` +- `extent`).  For the
/// category const_velocity, `aux` is the collider's material velocity.
struct MakeZSLevelSet : INode {
  void apply() override {
    auto ls = std::make_shared<ZenoLevelSet>();
    ls->dx = get_input2<float>("dx");
    ls->transferScheme = get_input2<std::string>("transfer");
    ls->category = get_input2<std::string>("category");
    const std::string &ts = ls->transferScheme;
    if (ts != "unknown" && ts != "apic" && ts != "flip" && ts != "aflip" && ts != "boundary")
      throw std::runtime_error("MakeZSLevelSet: unrecognized transfer scheme [" + ts + "]");
    const std::string &cat = ls->category;
    if (cat != "cellcentered" && cat != "collocated" && cat != "staggered" && cat != "const_velocity")
      throw std::runtime_error("MakeZSLevelSet: unknown levelset (grid) category [" + cat + "]");
    if (!(ls->dx > 0.f)) throw std::runtime_error("MakeZSLevelSet: dx must be positive");
    if (cat == "const_velocity" && has_input<NumericObject>("aux"))
      ls->const_vel = get_input<NumericObject>("aux")->get<vec3f>();
    const float h = ls->dx;
    if (has_input<PrimitiveObject>("sdf_prim")) {
      auto prim = get_input<PrimitiveObject>("sdf_prim");
      const vec3f d = get_input<NumericObject>("dims")->get<vec3f>();
      long long cells = 1;
      for (int a = 0; a < 3; ++a) {
        ls->dims[a] = (int)std::lround(d[a]);
        if (ls->dims[a] < 2) throw std::runtime_error("MakeZSLevelSet: dims must be >= 2");
        cells *= ls->dims[a];
      }
      const auto &pos = prim_access::pos(*prim);
      const auto *sdf = prim_access::float_attr(*prim, "sdf");
      if (!sdf || (long long)sdf->size() != cells || (long long)pos.size() != cells)
        throw std::runtime_error("MakeZSLevelSet: sdf_prim needs dims[0]*dims[1]*dims[2] "
                                 "vertices with a float attribute \"sdf\"");
      ls->origin = pos[0];
      ls->sdf = *sdf;
      if (auto *v = prim_access::vel(*prim, false); v && (long long)v->size() == cells) {
        ls->vel.resize(3 * cells);
        for (long long i = 0; i < cells; ++i)
          for (int a = 0; a < 3; ++a) ls->vel[a * cells + i] = (*v)[i][a];
      }
    } else {
      const std::string shape = get_input2<std::string>("shape");
      vec3f c{0.f, 0.f, 0.f};
      if (has_input<NumericObject>("center")) c = get_input<NumericObject>("center")->get<vec3f>();
      float half = 0.f;
      if (shape == "sphere")
        half = get_input2<float>("radius") + 3.f * h;
      else if (shape == "plane")
        half = get_input2<float>("extent");
      else
        throw std::runtime_error("MakeZSLevelSet: give sdf_prim or an analytic shape "
                                 "(sphere, plane)");
      const int n = (int)std::ceil(half / h);
      for (int a = 0; a < 3; ++a) {
        ls->dims[a] = 2 * n + 1;
        ls->origin[a] = c[a] - n * h;
      }
      const float r = get_input2<float>("radius"), y0 = get_input2<float>("height");
      const int m = 2 * n + 1;
      ls->sdf.resize((size_t)m * m * m);
      for (int k = 0; k < m; ++k)
        for (int j = 0; j < m; ++j)
          for (int i = 0; i < m; ++i) {
            const float p[3] = {ls->origin[0] + i * h, ls->origin[1] + j * h, ls->origin[2] + k * h};
            float v;
            if (shape == "sphere")
              v = std::sqrt((p[0] - c[0]) * (p[0] - c[0]) + (p[1] - c[1]) * (p[1] - c[1]) +
                            (p[2] - c[2]) * (p[2] - c[2])) - r;
            else
              v = p[1] - y0;
            ls->sdf[((size_t)k * m + j) * m + i] = v;
          }
    }
    set_output("ZSLevelSet", std::move(ls));
  }
};
ZENDEFNODE(MakeZSLevelSet, {
                               {{"float", "dx", "0.1"},
                                "aux",
                                {"enum unknown apic flip aflip boundary", "transfer", "unknown"},
                                {"enum cellcentered collocated staggered const_velocity",
                                 "category", "cellcentered"},
                                "sdf_prim",
                                "dims",
                                {"enum none sphere plane", "shape", "none"},
                                "center",
                                {"float", "radius", "0.1"},
                                {"float", "height", "0"},
                                {"float", "extent", "0.5"}},
                               {"ZSLevelSet"},
                               {},
                               {"SOP"},
                           });

/// ToZSBoundary (Generation.cu:1597-1647).  With a ZSLevelSet input the
/// boundary is that level-set collider under translation (+ rate), scale
/// (+ rate) and yaw-pitch-roll angles in degrees, attached to the context
/// by the first ApplyBoundaryOnZSGrid that uses it.  Without one, the
/// boundary is the analytic walls of the domain box [domain_min,
/// domain_max] (node indices from world coordinates / dx), `thickness`
/// cells thick (the additive inputs).
struct ToZSBoundary : INode {
  void apply() override {
    auto b = std::make_shared<ZenoBoundary>();
    const std::string type = get_input2<std::string>("type");
    int t = MPM_BC_STICKY;  // the reference's fallback (Generation.cu:1611)
    if (type == "slip" || type == "Slip")
      t = MPM_BC_SLIP;
    else if (type == "separate" || type == "Separate")
      t = MPM_BC_SEPARATE;
    if (has_input<ZenoLevelSet>("ZSLevelSet")) {
      b->ls = get_input<ZenoLevelSet>("ZSLevelSet");
      mpm_collider_desc &c = b->col;
      c = mpm_collider_desc{};
      c.type = t;
      c.scene = -1;
      c.scale = 1.0f;
      auto vec = [&](const char *k, float (&dst)[3]) {
        if (has_input<NumericObject>(k)) {
          const vec3f v = get_input<NumericObject>(k)->get<vec3f>();
          for (int a = 0; a < 3; ++a) dst[a] = v[a];
        }
      };
      vec("translation", c.translation);
      vec("translation_rate", c.translation_rate);
      vec("ypr_angles", c.ypr_deg);
      if (has_input<NumericObject>("scale")) c.scale = get_input<NumericObject>("scale")->get<float>();
      if (has_input<NumericObject>("scale_rate"))
        c.scale_rate = get_input<NumericObject>("scale_rate")->get<float>();
      b->bc.type = MPM_BC_NONE;
      set_output("ZSBoundary", b);
      return;
    }
    b->bc.type = t;
    b->bc.thickness = get_input2<int>("thickness");
    const float dx = get_input2<float>("dx");
    vec3f lo{0.f, 0.f, 0.f}, hi{1.f, 1.f, 1.f};
    if (has_input<NumericObject>("domain_min")) lo = get_input<NumericObject>("domain_min")->get<vec3f>();
    if (has_input<NumericObject>("domain_max")) hi = get_input<NumericObject>("domain_max")->get<vec3f>();
    for (int d = 0; d < 3; ++d) {
      b->bc.lo[d] = (int)std::lround(lo[d] / dx);
      b->bc.hi[d] = (int)std::lround(hi[d] / dx);
    }
    set_output("ZSBoundary", b);
  }
};
ZENDEFNODE(ToZSBoundary, {
                             {"ZSLevelSet",
                              "translation",
                              "translation_rate",
                              "scale",
                              "scale_rate",
                              "ypr_angles",
                              {"string", "type", "sticky"},
                              {"float", "dx", "0.1"},
                              {"int", "thickness", "3"},
                              "domain_min",
                              "domain_max"},
                             {"ZSBoundary"},
                             {},
                             {"MPM"},
                         });

/// ApplyBoundaryOnZSGrid (Boundary.cu:83-163)
struct ApplyBoundaryOnZSGrid : INode {
  void apply() override {
    auto grid = get_input<ZenoGrid>("ZSGrid");
    if (has_input<ZenoBoundary>("ZSBoundary")) {
      auto table = get_input<ZenoPartition>("ZSPartition");
      auto ctx = bound_ctx(table, "ApplyBoundaryOnZSGrid");
      auto b = get_input<ZenoBoundary>("ZSBoundary");
      attach_boundary(ctx, *b);
      // this boundary only: the walls, or this level set's collider
      if (b->ls)
        check(mpm_apply_collider(ctx->h, b->collider_id), "mpm_apply_collider");
      else
        check(mpm_apply_walls(ctx->h), "mpm_apply_walls");
    }
    set_output("ZSGrid", grid);
  }
};
ZENDEFNODE(ApplyBoundaryOnZSGrid, {
                                      {"ZSPartition", "ZSGrid", "ZSBoundary"},
                                      {"ZSGrid"},
                                      {},
                                      {"MPM"},
                                  });

/// ToBoundaryParticles (Generation.cpp:1154-1482): a triangle mesh to
/// boundary points -- its vertices (mass a third of their triangles' area in
/// dx^2, the primitive's "vel" or zero) and one point per triangle (its area,
/// centroid, mean velocity and unit normal).  Sprayed points (prim_tris) are
/// not supported.
struct ToBoundaryParticles : INode {
  void apply() override {
    auto prim = get_input<PrimitiveObject>("prim");
    if (has_input("prim_tris"))
      throw std::runtime_error("ToBoundaryParticles: sprayed particles (prim_tris) are not "
                               "implemented by this backend");
    const auto &pos = prim_access::pos(*prim);
    const auto &tris = prim_access::tris(*prim);
    if (tris.empty()) throw std::runtime_error("boundary primitive is not a surface mesh!");
    const float dx = get_input2<float>("dx");
    auto out = std::make_shared<ZenoParticles>();
    out->prim = prim;
    out->boundary = true;
    out->bdx = dx;
    const int64_t nv = (int64_t)pos.size(), nt = (int64_t)tris.size();
    std::vector<float> p(3 * nv), vel;
    std::vector<int32_t> t(3 * nt);
    for (int64_t i = 0; i < nv; ++i)
      for (int d = 0; d < 3; ++d) p[3 * i + d] = pos[i][d];
    for (int64_t i = 0; i < nt; ++i)
      for (int d = 0; d < 3; ++d) t[3 * i + d] = tris[i][d];
    if (auto *v = prim_access::vel(*prim, false); v && (int64_t)v->size() == nv) {
      vel.resize(3 * nv);
      for (int64_t i = 0; i < nv; ++i)
        for (int d = 0; d < 3; ++d) vel[3 * i + d] = (*v)[i][d];
    }
    out->b_verts = nv;
    out->b_n = nv + nt;
    out->bx.resize(3 * out->b_n);
    out->bv.resize(3 * out->b_n);
    out->bnrm.resize(3 * out->b_n);
    out->bm.resize(out->b_n);
    check(mpm_boundary_points_from_mesh(nv, p.data(), vel.empty() ? nullptr : vel.data(), nt,
                                        t.data(), dx, out->bx.data(), out->bv.data(),
                                        out->bm.data(), out->bnrm.data()),
          "mpm_boundary_points_from_mesh");
    set_output("ZSParticles", out);
  }
};
ZENDEFNODE(ToBoundaryParticles, {
                                    {"prim", "prim_tris", {"float", "dx", "0.1"}},
                                    {"ZSParticles"},
                                    {},
                                    {"MPM"},
                                });

/// ZSBoundaryPrimitiveToZSGrid (Transfer.cu:1532-1623): the boundary points
/// into a grid of transfer "boundary" (scattered, with the linear kernel, in
/// the context of the particles the grid is applied to)
struct ZSBoundaryPrimitiveToZSGrid : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    auto grid = get_input<ZenoGrid>("ZSGrid");
    (void)get_input<ZenoPartition>("ZSPartition");
    if (grid->transferScheme != "boundary") throw std::runtime_error("grid is not of boundary type!");
    if (!pars->boundary)
      throw std::runtime_error("boundary primitive does not have normal channel!");
    grid->bnd = pars;
    set_output("ZSGrid", grid);
  }
};
ZENDEFNODE(ZSBoundaryPrimitiveToZSGrid, {
                                            {"ZSParticles", "ZSPartition", "ZSGrid"},
                                            {"ZSGrid"},
                                            {},
                                            {"MPM"},
                                        });

/// ApplyGridBoundaryOnZSGrid (Boundary.cu:18-69): the boundary grid's
/// velocity on every node of the grid whose mass, and whose boundary node's
/// mass, is non-zero -- sticky, slip or separate along the boundary normal.
/// The boundary grid is built in the particles' context the first time (and
/// again when its points or the type change).
struct ApplyGridBoundaryOnZSGrid : INode {
  void apply() override {
    auto grid = get_input<ZenoGrid>("ZSGrid");
    auto table = get_input<ZenoPartition>("ZSPartition");
    auto bg = get_input<ZenoGrid>("BoundaryZSGrid");
    (void)get_input<ZenoPartition>("BoundaryZSPartition");
    if (bg->transferScheme != "boundary")
      throw std::runtime_error("boundary grid is not of boundary type!");
    if (!bg->bnd)
      throw std::runtime_error("ApplyGridBoundaryOnZSGrid: the boundary grid holds no points "
                               "(run ZSBoundaryPrimitiveToZSGrid first)");
    auto ctx = bound_ctx(table, "ApplyGridBoundaryOnZSGrid");
    const std::string ts = get_param<std::string>("type");
    const int32_t type = ts == "sticky" ? MPM_BC_STICKY : (ts == "slip" ? MPM_BC_SLIP : MPM_BC_SEPARATE);
    const ZenoParticles &b = *bg->bnd;
    if (std::fabs(b.bdx - ctx->dx) > 1e-6f * ctx->dx)
      throw std::runtime_error("the boundary particles' dx differs from the grid's");
    if (ctx->bnd_src != (const void *)&b || ctx->bnd_type != type) {
      check(mpm_set_grid_boundary(ctx->h, type, b.b_verts, b.b_n - b.b_verts, b.bx.data(),
                                  b.bv.data(), b.bm.data(), b.bnrm.data()),
            "mpm_set_grid_boundary");
      ctx->bnd_src = &b;
      ctx->bnd_type = type;
    }
    check(mpm_apply_grid_boundary(ctx->h), "mpm_apply_grid_boundary");
    set_output("ZSGrid", grid);
  }
};
ZENDEFNODE(ApplyGridBoundaryOnZSGrid, {
                                          {"ZSPartition", "ZSGrid", "BoundaryZSPartition",
                                           "BoundaryZSGrid"},
                                          {"ZSGrid"},
                                          {{"enum sticky slip separate", "type", "sticky"}},
                                          {"MPM"},
                                      });

/// StepZSBoundary (Generation.cu:1662-1685): b += db/dt dt, s += ds/dt dt,
/// on the boundary and, once attached, on its collider in the context
struct StepZSBoundary : INode {
  void apply() override {
    auto b = get_input<ZenoBoundary>("ZSBoundary");
    const float dt = get_input2<float>("dt");
    b->col.scale += b->col.scale_rate * dt;
    for (int a = 0; a < 3; ++a) b->col.translation[a] += b->col.translation_rate[a] * dt;
    if (auto ctx = b->attached.lock(); ctx && b->collider_id >= 0)
      check(mpm_step_colliders(ctx->h, b->collider_id, dt), "mpm_step_colliders");
    set_output("ZSBoundary", b);
  }
};
ZENDEFNODE(StepZSBoundary, {
                               {"ZSBoundary", {"float", "dt", "0"}},
                               {"ZSBoundary"},
                               {},
                               {"MPM"},
                           });

/// ComputeVonMises (Generation.cu:1873-1920): the von Mises stress of the
/// StVK-Hencky particles into their "vms" attribute (log10(vms + 1) by
/// default).
struct ComputeVonMises : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    const int option = get_param<int>("by_log1p(base10)");
    check(mpm_compute_von_mises(pars->ctx->h, option), "mpm_compute_von_mises");
    set_output("ZSParticles", pars);
  }
};
ZENDEFNODE(ComputeVonMises, {
                                {"ZSParticles"},
                                {"ZSParticles"},
                                {{"int", "by_log1p(base10)", "1"}},
                                {"MPM"},
                            });

/// WriteZSParticles (Generation.cu:1842-1871): the particles' positions and
/// their von Mises stress ("vms", from ComputeVonMises; 0 before it) as a
/// point file at `path`, in upload order.  The reference writes through
/// Partio (absent here); this writes the Houdini classic ASCII geometry
/// format (".geo": the PGEOMETRY V5 header, a float point attribute
/// "stress", one "x y z 1 (stress)" line per point), which Partio and
/// Houdini read.  Other extensions are refused.
struct WriteZSParticles : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    const std::string path = get_input2<std::string>("path");
    if (path.size() < 4 || path.compare(path.size() - 4, 4, ".geo") != 0)
      throw std::runtime_error("WriteZSParticles: only the ASCII .geo format is written "
                               "(path '" + path + "')");
    if (!pars->ctx || pars->cloth || pars->tracker)
      throw std::runtime_error("WriteZSParticles: the input holds no MPM particles");
    const int64_t n = pars->n;
    std::vector<float> x(3 * n), vms(n);
    check(mpm_particles_download(pars->ctx->h, x.data(), nullptr, nullptr, nullptr, nullptr),
          "mpm_particles_download");
    check(mpm_particles_get_attr(pars->ctx->h, "vms", vms.data()), "mpm_particles_get_attr");
    std::FILE *f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("WriteZSParticles: cannot open '" + path + "'");
    std::fprintf(f, "PGEOMETRY V5\nNPoints %lld NPrims 0\nNPointGroups 0 NPrimGroups 0\n",
                 (long long)n);
    std::fprintf(f, "NPointAttrib 1 NVertexAttrib 0 NPrimAttrib 0 NAttrib 0\n");
    std::fprintf(f, "PointAttrib\nstress 1 float 0\n");
    for (int64_t i = 0; i < n; ++i)
      std::fprintf(f, "%.9g %.9g %.9g 1 (%.9g)\n", x[3 * i], x[3 * i + 1], x[3 * i + 2], vms[i]);
    std::fprintf(f, "beginExtra\nendExtra\n");
    const bool ok = std::fclose(f) == 0;
    if (!ok) throw std::runtime_error("WriteZSParticles: writing '" + path + "' failed");
  }
};
ZENDEFNODE(WriteZSParticles, {
                                 {"ZSParticles", {"string", "path", ""}},
                                 {},
                                 {},
                                 {"MPM"},
                             });

/// ComputeParticleBeta (Boundary.cu:172-516): beta for the AFLIP position
/// update.  With a level-set ZSBoundary, particles that at x + dt v are
/// inside it and move into it get 0; otherwise 0.5 where det F > 1, else 0.
/// A ZSBoundary of box walls (no level set) gives the volume criterion only;
/// a boundary grid (transfer "boundary") the test against its nodes at
/// x + dt v (Boundary.cu:172-222).
struct ComputeParticleBeta : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    auto ctx = pars->ctx;
    int32_t collider = -1;
    if (has_input<ZenoGrid>("ZSBoundary(Grid)")) {  // a boundary grid
      auto bg = get_input<ZenoGrid>("ZSBoundary(Grid)");
      if (bg->transferScheme != "boundary" || !bg->bnd)
        throw std::runtime_error("ComputeParticleBeta: the ZSGrid is not a filled boundary grid");
      const ZenoParticles &b = *bg->bnd;
      if (ctx->bnd_src != (const void *)&b) {  // built as ApplyGridBoundaryOnZSGrid would
        const int32_t type = ctx->bnd_src ? ctx->bnd_type : MPM_BC_STICKY;
        check(mpm_set_grid_boundary(ctx->h, type, b.b_verts, b.b_n - b.b_verts, b.bx.data(),
                                    b.bv.data(), b.bm.data(), b.bnrm.data()),
              "mpm_set_grid_boundary");
        ctx->bnd_src = &b;
        ctx->bnd_type = type;
      }
      collider = -2;
    }
    if (has_input<ZenoBoundary>("ZSBoundary(Grid)")) {
      auto b = get_input<ZenoBoundary>("ZSBoundary(Grid)");
      if (b->ls) {
        attach_boundary(ctx, *b);
        collider = b->collider_id;
      }
    }
    check(mpm_compute_particle_beta(ctx->h, get_dt(*this), collider), "mpm_compute_particle_beta");
    set_output("ZSParticles", pars);
  }
};
ZENDEFNODE(ComputeParticleBeta, {
                                    {"ZSParticles", "ZSPartition", "ZSBoundary(Grid)", "dt"},
                                    {"ZSParticles"},
                                    {},
                                    {"MPM"},
                                });

/// ZSGridToZSParticle (Transfer.cu:1069-1173)
struct ZSGridToZSParticle : INode {
  void apply() override {
    auto grid = get_input<ZenoGrid>("ZSGrid");
    auto table = get_input<ZenoPartition>("ZSPartition");
    auto pars = get_input<ZenoParticles>("ZSParticles");
    auto ctx = bound_ctx(table, "ZSGridToZSParticle");
    if (pars->ctx != ctx) throw std::runtime_error("ZSParticles and ZSPartition are not bound");
    (void)grid;
    check(mpm_g2p(ctx->h, get_dt(*this)), "mpm_g2p");
    table->rebuilt = false;
    set_output("ZSParticles", pars);
  }
};
ZENDEFNODE(ZSGridToZSParticle, {
                                   {"ZSGrid", "ZSPartition", "ZSParticles", "dt"},
                                   {"ZSParticles"},
                                   {},
                                   {"MPM"},
                               });

/// ZSReturnMapping (MPMPipeline.cu:953-1138): Drucker-Prager projection
struct ZSReturnMapping : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    check(mpm_return_mapping(pars->ctx->h), "mpm_return_mapping");
    set_output("ZSParticles", pars);
  }
};
ZENDEFNODE(ZSReturnMapping, {
                                {"ZSParticles"},
                                {"ZSParticles"},
                                {},
                                {"MPM"},
                            });

/// AdjustParticleMaterial (Temp.cu:16-56): per-particle E, nu blended along
/// one axis between (end_soft, E_soft, nu_soft) and (end_hard, E_hard, nu_hard)
struct AdjustParticleMaterial : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    const float Eh = get_input2<float>("E_hard"), Es = get_input2<float>("E_soft");
    const float nh = get_input2<float>("nu_hard"), ns = get_input2<float>("nu_soft");
    const float eh = get_input2<float>("end_hard"), es = get_input2<float>("end_soft");
    const std::string orient = get_param<std::string>("orientation");
    const int d = orient == "x" ? 0 : (orient == "y" ? 1 : 2);
    const int64_t n = pars->n;
    std::vector<float> x(3 * n), mu(n), lam(n);
    check(mpm_particles_download(pars->ctx->h, x.data(), nullptr, nullptr, nullptr, nullptr),
          "mpm_particles_download");
    const float span = eh - es;
    for (int64_t i = 0; i < n; ++i) {
      const float ratio = std::min(1.0f, std::max(0.0f, (eh - x[3 * i + d]) / span));
      const float E = Es * ratio + Eh * (1.0f - ratio);
      const float nu = ns * ratio + nh * (1.0f - ratio);
      mu[i] = E / (2.0f * (1.0f + nu));
      lam[i] = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
    }
    check(mpm_particles_set_lame(pars->ctx->h, mu.data(), lam.data()), "mpm_particles_set_lame");
    set_output("ZSParticles", pars);
  }
};
ZENDEFNODE(AdjustParticleMaterial, {
                                       {"ZSParticles",
                                        {"float", "E_hard", "100"},
                                        {"float", "E_soft", "50"},
                                        {"float", "nu_hard", "0.4"},
                                        {"float", "nu_soft", "0.2"},
                                        {"float", "end_hard", "1"},
                                        {"float", "end_soft", "-0.5"}},
                                       {"ZSParticles"},
                                       {{"enum x y z", "orientation", "y"}},
                                       {"MPM"},
                                   });

/// UpdatePrimitiveFromZSParticles (Generation.cu:1088-1158): x, v back into
/// the source primitive ("pos", "vel")
struct UpdatePrimitiveFromZSParticles : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    if (pars->tracker) {  // the tracker points back into their primitive
      auto ctx = pars->tracker_ctx.lock();
      if (ctx && pars->prim) {
        auto &pos = prim_access::pos(*pars->prim);
        const int64_t n = (int64_t)pos.size();
        std::vector<float> x(3 * n), v(3 * n);
        check(mpm_trackers_download(ctx->h, x.data(), v.data()), "mpm_trackers_download");
        auto &vel = *prim_access::vel(*pars->prim, true);
        vel.resize(n);
        for (int64_t i = 0; i < n; ++i)
          for (int d = 0; d < 3; ++d) {
            pos[i][d] = x[3 * i + d];
            vel[i][d] = v[3 * i + d];
          }
      }
      set_output("ZSParticles", pars);
      return;
    }
    if (pars->cloth) {  // the cloth's vertices back into its mesh
      auto ctx = pars->cloth_ctx.lock();
      if (ctx && pars->prim) {
        auto &pos = prim_access::pos(*pars->prim);
        const int64_t n = (int64_t)pos.size();
        std::vector<float> x(3 * n), v(3 * n);
        check(mpm_cloth_download(ctx->h, x.data(), v.data(), nullptr, nullptr, nullptr, nullptr,
                                 nullptr, nullptr),
              "mpm_cloth_download");
        auto &vel = *prim_access::vel(*pars->prim, true);
        vel.resize(n);
        for (int64_t i = 0; i < n; ++i)
          for (int d = 0; d < 3; ++d) {
            pos[i][d] = x[3 * i + d];
            vel[i][d] = v[3 * i + d];
          }
      }
      set_output("ZSParticles", pars);
      return;
    }
    if (pars->prim) {
      const int64_t n = pars->n;
      std::vector<float> x(3 * n), v(3 * n);
      check(mpm_particles_download(pars->ctx->h, x.data(), v.data(), nullptr, nullptr, nullptr),
            "mpm_particles_download");
      auto &pos = prim_access::pos(*pars->prim);
      if ((int64_t)pos.size() != n) pos.resize(n);
      auto &vel = *prim_access::vel(*pars->prim, true);
      vel.resize(n);
      for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
          pos[i][d] = x[3 * i + d];
          vel[i][d] = v[3 * i + d];
        }
    }
    set_output("ZSParticles", pars);
  }
};
ZENDEFNODE(UpdatePrimitiveFromZSParticles, {
                                               {"ZSParticles"},
                                               {"ZSParticles"},
                                               {},
                                               {"MPM"},
                                           });

/// RetrievePrimitiveFromZSParticles (Generation.cu:1695-1715): the source
/// primitive the particles were made from (as the last write-back left it).
struct RetrievePrimitiveFromZSParticles : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    if (!pars->prim) throw std::runtime_error("there are no zsparticles!");
    set_output("prim", pars->prim);
  }
};
ZENDEFNODE(RetrievePrimitiveFromZSParticles, {
                                                 {"ZSParticles"},
                                                 {"prim"},
                                                 {},
                                                 {"MPM"},
                                             });

/// ExtractPrimitiveFromZSParticles (Generation.cu:1717-1742): the source
/// primitive, and the particle object emptied (its device context released
/// once no partition or grid holds it).
struct ExtractPrimitiveFromZSParticles : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    if (!pars->prim) throw std::runtime_error("there are no zsparticles!");
    auto prim = pars->prim;
    *pars = ZenoParticles();
    set_output("prim", prim);
  }
};
ZENDEFNODE(ExtractPrimitiveFromZSParticles, {
                                                {"ZSParticles"},
                                                {"prim"},
                                                {},
                                                {"MPM"},
                                            });

namespace {

// A particle channel of a ZSParticles object in upload order: its width
// (1 or 3) and values.  MPM particles: x, v and the scalar attributes of
// mpm_particles_get_attr; cloth and curve vertices ("vert") and elements
// ("quad"): x, v; tracker points: x, v.
int fetch_channel(ZenoParticles &pars, bool quad, const std::string &name,
                  std::vector<float> &out) {
  auto fail = [&]() -> int {
    throw std::runtime_error("the particles has no specified channel [" + name + "]");
  };
  if (name != "x" && name != "v" && (pars.cloth || pars.tracker || quad)) return fail();
  if (pars.cloth) {
    auto ctx = pars.cloth_ctx.lock();
    if (!ctx) throw std::runtime_error("the cloth is not attached to a context yet");
    const int64_t nv = (int64_t)prim_access::pos(*pars.prim).size();
    const int64_t ne = pars.cloth_desc.kind == MPM_MESH_CURVE
                           ? (int64_t)prim_access::lines(*pars.prim).size()
                           : (int64_t)prim_access::tris(*pars.prim).size();
    out.assign(3 * (quad ? ne : nv), 0.0f);
    float *dst = out.data();
    check(mpm_cloth_download(ctx->h, !quad && name == "x" ? dst : nullptr,
                             !quad && name == "v" ? dst : nullptr, nullptr,
                             quad && name == "x" ? dst : nullptr, quad && name == "v" ? dst : nullptr,
                             nullptr, nullptr, nullptr),
          "mpm_cloth_download");
    return 3;
  }
  if (pars.tracker) {
    auto ctx = pars.tracker_ctx.lock();
    if (!ctx) throw std::runtime_error("the trackers are not attached to a context yet");
    out.assign(3 * pars.n, 0.0f);
    check(mpm_trackers_download(ctx->h, name == "x" ? out.data() : nullptr,
                                name == "v" ? out.data() : nullptr),
          "mpm_trackers_download");
    return 3;
  }
  if (!pars.ctx) return fail();
  if (name == "x" || name == "v") {
    out.assign(3 * pars.n, 0.0f);
    check(mpm_particles_download(pars.ctx->h, name == "x" ? out.data() : nullptr,
                                 name == "v" ? out.data() : nullptr, nullptr, nullptr, nullptr),
          "mpm_particles_download");
    return 3;
  }
  static const std::set<std::string> scalars = {"J", "m", "vol", "vms", "beta", "mu", "lam"};
  if (!scalars.count(name)) return fail();
  out.assign(pars.n, 0.0f);
  check(mpm_particles_get_attr(pars.ctx->h, name.c_str(), out.data()), "mpm_particles_get_attr");
  return 1;
}

// the channel into the primitive's vertex (or triangle) attribute; x of the
// vertices becomes "pos"
void store_channel(PrimitiveObject &prim, bool quad, const std::string &name, int dim,
                   const std::vector<float> &v) {
  const std::string dst = (!quad && name == "x") ? "pos" : name;
  if (dim == 1) {
    auto &a = prim_access::attr<float>(prim, quad, dst);
    const size_t n = std::min(a.size(), v.size());
    for (size_t i = 0; i < n; ++i) a[i] = v[i];
  } else {
    auto &a = prim_access::attr<vec3f>(prim, quad, dst);
    const size_t n = std::min(a.size(), v.size() / 3);
    for (size_t i = 0; i < n; ++i) a[i] = vec3f{v[3 * i], v[3 * i + 1], v[3 * i + 2]};
  }
}

}  // namespace

/// UpdatePrimitiveAttributesFromZSParticles (Generation.cu:1165-1286): the
/// named channels (separated by any of " :;,.") into attributes of the
/// source primitive's vertices ("vert"; x becomes pos) or triangles ("quad",
/// the cloth's elements); channels must be scalars or 3-vectors.
struct UpdatePrimitiveAttributesFromZSParticles : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    const std::string tags = get_input2<std::string>("attrs");
    const bool quad = get_param<std::string>("location") == "quad";
    if (!pars->prim) throw std::runtime_error("there are no zsparticles!");
    std::set<std::string> names;
    const std::string seps = " :;,.";
    size_t st = tags.find_first_not_of(seps);
    while (st != std::string::npos) {
      const size_t ed = tags.find_first_of(seps, st);
      names.insert(tags.substr(st, ed == std::string::npos ? std::string::npos : ed - st));
      st = ed == std::string::npos ? ed : tags.find_first_not_of(seps, ed);
    }
    std::vector<float> buf;
    for (const auto &name : names) {
      const int dim = fetch_channel(*pars, quad, name, buf);
      store_channel(*pars->prim, quad, name, dim, buf);
    }
    set_output("ZSParticles", pars);
    set_output("prim", pars->prim);
  }
};
ZENDEFNODE(UpdatePrimitiveAttributesFromZSParticles, {
                                                         {"ZSParticles", {"string", "attrs", ""}},
                                                         {"ZSParticles", "prim"},
                                                         {{"enum vert quad", "location", "vert"}},
                                                         {"MPM"},
                                                     });

/// UpdatePrimitiveAttrFromZSParticles (Generation.cu:1288-1468): one channel
/// into a float or vec3f attribute of the source primitive's vertices or
/// triangles (the type must match the channel's width).
struct UpdatePrimitiveAttrFromZSParticles : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    const std::string name = get_input2<std::string>("attr");
    const std::string type = get_param<std::string>("type");
    const std::string location = get_param<std::string>("location");
    if (location != "vert" && location != "quad")
      throw std::runtime_error("UNRECOGINIZED LOCATION SPECIFIED");
    if (type != "float" && type != "vec3f") throw std::runtime_error("INVALID SPECIFIED TYPE");
    if (pars->prim) {
      std::vector<float> buf;
      const bool quad = location == "quad";
      const int dim = fetch_channel(*pars, quad, name, buf);
      if (dim != (type == "float" ? 1 : 3))
        throw std::runtime_error("UpdatePrimitiveAttrFromZSParticles: channel [" + name +
                                 "] has width " + std::to_string(dim) + ", not " + type);
      store_channel(*pars->prim, quad, name, dim, buf);
    }
    set_output("ZSParticles", pars);
  }
};
ZENDEFNODE(UpdatePrimitiveAttrFromZSParticles,
           {
               {"ZSParticles", {"string", "attr", "x"}},
               {"ZSParticles"},
               {{"enum float vec3f", "type", "vec3f"}, {"enum vert quad", "location", "vert"}},
               {"MPM"},
           });

/// ZSParticlesToPrimitiveObject (Generation.cu:1744-1833): a new primitive
/// with "pos" and "vel"
struct ZSParticlesToPrimitiveObject : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    const int64_t n = pars->n;
    std::vector<float> x(3 * n), v(3 * n);
    check(mpm_particles_download(pars->ctx->h, x.data(), v.data(), nullptr, nullptr, nullptr),
          "mpm_particles_download");
    auto prim = std::make_shared<PrimitiveObject>();
    auto &pos = prim_access::pos(*prim);
    pos.resize(n);
    auto &vel = *prim_access::vel(*prim, true);
    vel.resize(n);
    for (int64_t i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
        pos[i][d] = x[3 * i + d];
        vel[i][d] = v[3 * i + d];
      }
    set_output("prim", prim);
  }
};
ZENDEFNODE(ZSParticlesToPrimitiveObject, {
                                             {"ZSParticles"},
                                             {"prim"},
                                             {},
                                             {"MPM"},
                                         });

/// ZSMPMSubstep (new, additive): partition, grid, P2G, grid update +
/// boundary, G2P + return mapping for `substeps` substeps on the device in
/// one call (CUDA-graph replay, no host synchronisation between substeps).
struct ZSMPMSubstep : INode {
  void apply() override {
    auto pars = get_input<ZenoParticles>("ZSParticles");
    ensure_cloth_ctx(*pars);
    auto ctx = pars->ctx;
    float acc[3] = {0.0f, get_input2<float>("gravity"), 0.0f};
    if (has_input("Accel")) {
      auto a = get_input<NumericObject>("Accel")->get<vec3f>();
      acc[0] = a[0];
      acc[1] = a[1];
      acc[2] = a[2];
    }
    check(mpm_set_gravity(ctx->h, acc[0], acc[1], acc[2]), "mpm_set_gravity");
    if (has_input<ZenoBoundary>("ZSBoundary"))
      attach_boundary(ctx, *get_input<ZenoBoundary>("ZSBoundary"));
    // a level-set collider after the walls; the substeps advance it on the
    // device (b += db/dt dt, s += ds/dt dt at the start of each substep)
    if (has_input<ZenoBoundary>("ZSCollider"))
      attach_boundary(ctx, *get_input<ZenoBoundary>("ZSCollider"));
    if (has_input<ZenoParticles>("ZSCloth"))
      attach_cloth(ctx, *get_input<ZenoParticles>("ZSCloth"));
    if (has_input<ZenoParticles>("ZSTrackers"))
      attach_trackers(ctx, *get_input<ZenoParticles>("ZSTrackers"));
    if (has_input<ZenoParticles>("ZSBending"))
      attach_bending(ctx, *get_input<ZenoParticles>("ZSBending"));
    // the transfer scheme of a MakeZSGrid (default APIC)
    if (has_input<ZenoGrid>("BoundaryZSGrid")) {  // a boundary grid, every substep
      auto bg = get_input<ZenoGrid>("BoundaryZSGrid");
      if (bg->transferScheme != "boundary" || !bg->bnd)
        throw std::runtime_error("ZSMPMSubstep: BoundaryZSGrid is not a filled boundary grid");
      const std::string ts = get_input2<std::string>("boundary_type");
      const int32_t type =
          ts == "sticky" ? MPM_BC_STICKY : (ts == "slip" ? MPM_BC_SLIP : MPM_BC_SEPARATE);
      const ZenoParticles &b = *bg->bnd;
      if (ctx->bnd_src != (const void *)&b || ctx->bnd_type != type) {
        check(mpm_set_grid_boundary(ctx->h, type, b.b_verts, b.b_n - b.b_verts, b.bx.data(),
                                    b.bv.data(), b.bm.data(), b.bnrm.data()),
              "mpm_set_grid_boundary");
        ctx->bnd_src = &b;
        ctx->bnd_type = type;
      }
    }
    if (has_input<ZenoGrid>("ZSGrid"))
      check(mpm_set_transfer(ctx->h, transfer_of(*get_input<ZenoGrid>("ZSGrid"))),
            "mpm_set_transfer");
    check(mpm_substep(ctx->h, get_dt(*this), get_input2<int>("substeps")), "mpm_substep");
    mpm_stats st{};
    check(mpm_get_stats(ctx->h, &st), "mpm_get_stats");
    check(st.status, "substep");
    set_output("ZSParticles", pars);
    set_output("MaxVelSqr", std::make_shared<NumericObject>(st.max_vel_sqr));
  }
};
ZENDEFNODE(ZSMPMSubstep, {
                             {"ZSParticles",
                              "ZSBoundary",
                              "ZSCollider",
                              "ZSGrid",
                              "ZSCloth",
                              "ZSTrackers",
                              "ZSBending",
                              "BoundaryZSGrid",
                              {"enum sticky slip separate", "boundary_type", "sticky"},
                              "dt",
                              {"float", "gravity", "-9.8"},
                              "Accel",
                              {"int", "substeps", "1"}},
                             {"ZSParticles", "MaxVelSqr"},
                             {},
                             {"MPM"},
                         });

}  // namespace zeno
