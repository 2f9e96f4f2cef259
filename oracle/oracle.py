"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check and bench.py's CPU legs import this module; the
product path (zeno_gb300/) never does.  The oracle restates the reference's
CuLagrange MLS-MPM substep (see mpm_oracle.cpp for the file:line of every
node body it follows).  Parity with reference outputs is unpinned: the
reference ships no MPM golden vectors and its substep cannot run without the
absent zpc submodule.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libzsmpm_oracle.so")


class OrcMaterial(C.Structure):
    _fields_ = [("type", C.c_int32), ("plasticity", C.c_int32), ("E", C.c_float),
                ("nu", C.c_float), ("density", C.c_float), ("friction_angle_deg", C.c_float),
                ("bulk", C.c_float), ("gamma", C.c_float), ("yield_stress", C.c_float),
                ("cc_beta", C.c_float), ("cc_xi", C.c_float)]


class OrcCollider(C.Structure):
    _fields_ = [("type", C.c_int32), ("dims", C.c_int32 * 3), ("origin", C.c_float * 3),
                ("spacing", C.c_float), ("sdf", C.c_void_p), ("velocity", C.c_void_p),
                ("const_velocity", C.c_float * 3), ("translation", C.c_float * 3),
                ("translation_rate", C.c_float * 3), ("scale", C.c_float),
                ("scale_rate", C.c_float), ("ypr_deg", C.c_float * 3)]


class OrcCloth(C.Structure):
    _fields_ = [("kind", C.c_int32), ("model", C.c_int32), ("gamma", C.c_float), ("k", C.c_float),
                ("fa", C.c_float),
                ("dc", C.c_float), ("n_verts", C.c_int64), ("n_eles", C.c_int64)] + \
               [(k, C.c_void_p) for k in ("vx", "vv", "vC", "vm", "ex", "ev", "eC", "eF", "ed",
                                          "eDmInv", "em", "evol", "emu", "elam", "inds")] + \
               [("n_springs", C.c_int64), ("spring_v", C.c_void_p), ("spring_k", C.c_void_p),
                ("spring_rl", C.c_void_p), ("thickness", C.c_double), ("vbeta", C.c_void_p)]


CLOTH_VERT = {"vx": 3, "vv": 3, "vC": 9, "vm": 1}
CLOTH_ELE = {"ex": 3, "ev": 3, "eC": 9, "eF": 9, "ed": 9, "eDmInv": 9, "em": 1, "evol": 1,
             "emu": 1, "elam": 1}


class OrcTrackers(C.Structure):
    _fields_ = [("n", C.c_int64), ("x", C.c_void_p), ("v", C.c_void_p)]


class OrcGridBoundary(C.Structure):
    _fields_ = [("type", C.c_int32), ("n_verts", C.c_int64), ("n_eles", C.c_int64),
                ("x", C.c_void_p), ("v", C.c_void_p), ("m", C.c_void_p), ("nrm", C.c_void_p)]


class OrcScene(C.Structure):
    _fields_ = [("dx", C.c_float), ("gravity", C.c_float * 3), ("block_lo", C.c_int32 * 3),
                ("block_dims", C.c_int32 * 3), ("bc_type", C.c_int32),
                ("bc_thickness", C.c_int32), ("bc_lo", C.c_int32 * 3), ("bc_hi", C.c_int32 * 3),
                ("n_materials", C.c_int32), ("materials", C.POINTER(OrcMaterial)),
                ("n_colliders", C.c_int32), ("colliders", C.POINTER(OrcCollider)),
                ("collider_autostep", C.c_int32), ("transfer", C.c_int32),
                ("cloth", C.POINTER(OrcCloth)), ("trackers", C.POINTER(OrcTrackers)),
                ("grid_boundary", C.POINTER(OrcGridBoundary))]


class OrcStats(C.Structure):
    _fields_ = [("max_vel_sqr", C.c_double), ("n_pblocks", C.c_int64),
                ("n_gblocks", C.c_int64), ("status", C.c_int32)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f))
                                             for f in ("mpm_oracle.cpp", "mpm_oracle.h")):
        subprocess.run(["make", "-s", "-C", HERE, "-B"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_partition.argtypes = [C.POINTER(OrcScene), C.c_int64, P, C.c_int64, P, P, P, P,
                                    C.c_int64, P, P]
        L.orc_partition.restype = C.c_int32
        for name, real in (("orc_run_f64", C.c_double), ("orc_run_f32", C.c_float)):
            f = getattr(L, name)
            f.argtypes = [C.POINTER(OrcScene), C.c_int64] + [P] * 11 + [real, C.c_int32,
                                                                        C.c_int32,
                                                                        C.POINTER(OrcStats)]
            f.restype = C.c_int32
        L.orc_particle_beta_f64.argtypes = [C.POINTER(OrcScene), C.c_int64, P, P, P, P, P,
                                            C.c_double, C.c_int32, P]
        L.orc_particle_beta_f64.restype = C.c_int32
        L.orc_von_mises_f64.argtypes = [C.POINTER(OrcScene), C.c_int64, P, P, C.c_int32, P]
        L.orc_von_mises_f64.restype = C.c_int32
        L.orc_cloth_init_f64.argtypes = [C.c_int64, P, P, C.c_int64, P, C.c_float, C.c_float,
                                         C.c_float, C.c_float, C.POINTER(OrcCloth)]
        L.orc_cloth_init_f64.restype = C.c_int32
        L.orc_curve_init_f64.argtypes = L.orc_cloth_init_f64.argtypes
        L.orc_curve_init_f64.restype = C.c_int32
        L.orc_cloth_beta_f64.argtypes = [C.POINTER(OrcScene), C.POINTER(OrcCloth), C.c_double,
                                         C.c_int32]
        L.orc_cloth_beta_f64.restype = C.c_int32
        L.orc_sym_eig3.argtypes = [P, P, P]
        L.orc_kirchhoff.argtypes = [C.POINTER(OrcMaterial), P, C.c_double, P]
        L.orc_kirchhoff.restype = C.c_int32
        L.orc_project_dp.argtypes = [C.POINTER(OrcMaterial), P]
        L.orc_project_dp.restype = C.c_int32
        L.orc_project_hencky.argtypes = [C.POINTER(OrcMaterial), P, P]
        L.orc_project_hencky.restype = C.c_int32
        L.orc_max_threads.restype = C.c_int32
        L.orc_boundary_points_from_mesh.argtypes = [C.c_int64, P, P, C.c_int64, P, C.c_float,
                                                    P, P, P, P]
        L.orc_boundary_points_from_mesh.restype = C.c_int32
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def make_material(m) -> OrcMaterial:
    return OrcMaterial(int(m.type), int(m.plasticity), float(m.E), float(m.nu),
                       float(m.density), float(m.friction_angle_deg), float(m.bulk),
                       float(m.gamma), float(getattr(m, "yield_stress", 1e5)),
                       float(getattr(m, "cc_beta", 2.0)), float(getattr(m, "cc_xi", 1.0)))


class _SceneHolder:
    def __init__(self, scene):
        mats = (OrcMaterial * max(1, len(scene.materials)))(
            *[make_material(m) for m in scene.materials])
        self.mats = mats
        cols = list(getattr(scene, "colliders", []) or [])
        self.arrays = []  # keeps the sample grids alive

        def arr(a):
            a = np.ascontiguousarray(a, dtype=np.float32)
            self.arrays.append(a)
            return a.ctypes.data

        carr = (OrcCollider * max(1, len(cols)))()
        for i, c in enumerate(cols):
            nz, ny, nx = c.sdf.shape
            carr[i] = OrcCollider(int(c.type), (C.c_int32 * 3)(nx, ny, nz),
                                  (C.c_float * 3)(*c.origin), float(c.spacing), arr(c.sdf),
                                  arr(c.velocity) if c.velocity is not None else None,
                                  (C.c_float * 3)(*c.const_velocity),
                                  (C.c_float * 3)(*c.translation),
                                  (C.c_float * 3)(*c.translation_rate), float(c.scale),
                                  float(c.scale_rate), (C.c_float * 3)(*c.ypr_deg))
        self.cols = carr
        self.s = OrcScene(float(scene.dx), (C.c_float * 3)(*scene.gravity),
                          (C.c_int32 * 3)(*scene.block_lo), (C.c_int32 * 3)(*scene.block_dims),
                          int(scene.bc_type), int(scene.bc_thickness),
                          (C.c_int32 * 3)(*scene.bc_lo), (C.c_int32 * 3)(*scene.bc_hi),
                          len(scene.materials), C.cast(mats, C.POINTER(OrcMaterial)),
                          len(cols), C.cast(carr, C.POINTER(OrcCollider)), 1,
                          int(getattr(scene, "transfer", 0)), None, None, None)
        gbd = getattr(scene, "grid_boundary", None)
        if gbd is not None:
            self.gbd = OrcGridBoundary(int(gbd.type), int(gbd.n_verts),
                                       int(len(gbd.m) - gbd.n_verts), arr(gbd.x), arr(gbd.v),
                                       arr(gbd.m), arr(gbd.nrm))
            self.s.grid_boundary = C.pointer(self.gbd)

    def attach_cloth(self, cl: "OrcCloth"):
        self.cloth = cl
        self.s.cloth = C.pointer(cl)

    def attach_trackers(self, tk: "OrcTrackers"):
        self.trackers = tk
        self.s.trackers = C.pointer(tk)


def partition(scene, x: np.ndarray) -> dict:
    """Bit-exact reference partition of float32 positions x (n, 3)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n = x.shape[0]
    h = _SceneHolder(scene)
    D = int(np.prod(scene.block_dims))
    cap_pb = min(D, max(n, 1))
    cap_gb = D
    n_pb = np.zeros(1, np.int32)
    n_gb = np.zeros(1, np.int32)
    pb_dir = np.zeros(cap_pb, np.int32)
    pb_count = np.zeros(cap_pb, np.int32)
    perm = np.zeros(max(n, 1), np.int64)
    gb_dir = np.zeros(cap_gb, np.int32)
    rc = lib().orc_partition(C.byref(h.s), n, _ptr(x), cap_pb, _ptr(n_pb), _ptr(pb_dir),
                             _ptr(pb_count), _ptr(perm), cap_gb, _ptr(n_gb), _ptr(gb_dir))
    if rc != 0:
        raise RuntimeError(f"oracle partition failed with status {rc}")
    return {"pb_dir": pb_dir[:n_pb[0]].copy(), "pb_count": pb_count[:n_pb[0]].copy(),
            "perm": perm[:n].copy(), "gb_dir": gb_dir[:n_gb[0]].copy()}


def run(scene, parts, nsteps: int, precision: str = "f64", nthreads: int = 0,
        dt: float | None = None, inplace: bool = False):
    """Advance `parts` (a copy unless inplace) by nsteps substeps; returns
    (particles, stats).  inplace needs contiguous arrays of the precision."""
    dtype = np.float64 if precision == "f64" else np.float32
    p = parts if inplace else parts.copy(dtype=dtype)
    for k in ("x", "v", "C", "F", "J", "m", "vol", "mu", "lam", "beta"):
        a = getattr(p, k)
        if a is not None:
            if inplace and (a.dtype != dtype or not a.flags.c_contiguous):
                raise ValueError(f"in-place run needs contiguous {dtype.__name__} '{k}'")
            setattr(p, k, np.ascontiguousarray(a, dtype=dtype))
    p.mat = np.ascontiguousarray(p.mat, dtype=np.int32)
    h = _SceneHolder(scene)
    st = OrcStats()
    fn = lib().orc_run_f64 if precision == "f64" else lib().orc_run_f32
    rc = fn(C.byref(h.s), p.n, _ptr(p.x), _ptr(p.v), _ptr(p.C), _ptr(p.F), _ptr(p.J),
            _ptr(p.m), _ptr(p.vol), _ptr(p.mat), _ptr(p.mu), _ptr(p.lam), _ptr(p.beta),
            float(scene.dt if dt is None else dt), int(nsteps), int(nthreads), C.byref(st))
    stats = {"status": rc, "max_vel_sqr": st.max_vel_sqr, "n_pblocks": st.n_pblocks,
             "n_gblocks": st.n_gblocks}
    return p, stats


def particle_beta(scene, parts, dt: float | None = None, collider: int = -1) -> np.ndarray:
    """ComputeParticleBeta in FP64: beta per particle (upload order)."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    h = _SceneHolder(scene)
    x, v, F, J = f(parts.x), f(parts.v), f(parts.F), f(parts.J)
    mat = np.ascontiguousarray(parts.mat, dtype=np.int32)
    beta = np.zeros(parts.n)
    rc = lib().orc_particle_beta_f64(C.byref(h.s), parts.n, _ptr(x), _ptr(v), _ptr(F), _ptr(J),
                                     _ptr(mat), float(scene.dt if dt is None else dt),
                                     int(collider), _ptr(beta))
    if rc != 0:
        raise RuntimeError(f"oracle beta failed with status {rc}")
    return beta


def von_mises(scene, parts, by_log1p: bool = True, vms: np.ndarray | None = None) -> np.ndarray:
    """ComputeVonMises in FP64 (upload order); particles of other models keep
    the value in `vms` (default 0)."""
    F = np.ascontiguousarray(parts.F, dtype=np.float64)
    mat = np.ascontiguousarray(parts.mat, dtype=np.int32)
    out = np.zeros(parts.n) if vms is None else np.array(vms, dtype=np.float64)
    h = _SceneHolder(scene)
    rc = lib().orc_von_mises_f64(C.byref(h.s), parts.n, _ptr(F), _ptr(mat), int(by_log1p),
                                 _ptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle von Mises failed with status {rc}")
    return out


def _is_curve(mesh) -> bool:
    return np.asarray(mesh.tris).shape[1] == 2


def _cloth_struct(mesh, state, kind=None) -> OrcCloth:
    if mesh is None:  # the state alone (set-up free helpers)
        st = OrcCloth(int(kind), 0, 0.0, 0.0, 0.0, 0.0, int(state["vx"].shape[0]),
                      int(state["ex"].shape[0]))
    else:
        curve = _is_curve(mesh)
        st = OrcCloth(1 if curve else 0, 2 if curve else int(mesh.model), float(mesh.gamma),
                      float(mesh.k), float(mesh.fa), float(mesh.dc), int(state["vx"].shape[0]),
                      int(state["ex"].shape[0]))
    for k in list(CLOTH_VERT) + list(CLOTH_ELE) + ["inds"]:
        setattr(st, k, state[k].ctypes.data)
    if "spring_v" in state and len(state["spring_v"]):
        st.n_springs = int(state["spring_v"].shape[0])
        st.spring_v = state["spring_v"].ctypes.data
        st.spring_k = state["spring_k"].ctypes.data
        st.spring_rl = state["spring_rl"].ctypes.data
        st.thickness = float(state["thickness"])
    if "vbeta" in state:
        st.vbeta = state["vbeta"].ctypes.data
    return st


def cloth_beta(scene, state: dict, dt: float, collider: int = -1) -> np.ndarray:
    """ComputeParticleBeta on a triangle cloth state from cloth_init, in FP64
    (orc_cloth_beta_f64): sets and returns state["vbeta"], the per-vertex beta
    the FLIP-style vertex update then uses."""
    state["vbeta"] = np.zeros(state["vx"].shape[0])
    h = _SceneHolder(scene)
    st = _cloth_struct(None, state, kind=0)
    rc = lib().orc_cloth_beta_f64(C.byref(h.s), C.byref(st), float(dt), int(collider))
    if rc != 0:
        raise RuntimeError(f"oracle cloth beta failed with status {rc}")
    return state["vbeta"]


def cloth_bending(state: dict, stiffness: float, thickness: float, kind: str = "vertex") -> int:
    """ConstructBendingSprings (Generation.cu:563-1001) on a cloth state from
    cloth_init, in FP64, adding the springs to `state`; returns their count.
    Interior edges are found the reference's way: each triangle registers its
    directed edges (vi, vj) with vi < vj in its cyclic order (tri[2] -> tri[0]
    -> tri[1] -> tri[2]), and a directed edge vi -> vj with vi > vj whose
    reverse is registered by the neighbour becomes one pair.  "vertex": a
    spring between the edge's two opposite vertices, k = E / (24 (1 - nu^2))
    stiffness with the smaller E and nu of the two triangles (from their mu,
    lam), rest length their current distance.  "angle": the hinges exist in
    the reference but its force is identically zero (p2g_angle_bending_force,
    Transfer.cu:466-480: the angle is declared again inside a block and the
    outer one, 0, enters the force), so nothing is added.  "element" pairs are
    tagged as vertex springs without the vertex indices those read
    (Generation.cu:779, Transfer.cu:374): undefined, refused."""
    if kind == "element":
        raise ValueError("element bending springs are undefined in the reference")
    if kind not in ("vertex", "angle"):
        raise ValueError(f"unknown bending spring type {kind!r}")
    tris = np.asarray(state["inds"], dtype=np.int64)
    mu, lam = np.asarray(state["emu"]), np.asarray(state["elam"])
    E = mu * (3 * lam + 2 * mu) / (lam + mu)
    nu = lam / (2 * (lam + mu))
    edge_ele = {}
    for e, t in enumerate(tris):
        vi = int(t[2])
        for vj in t:
            vj = int(vj)
            if vi < vj:
                edge_ele[(vi, vj)] = e
            vi = vj
    pairs, ks = [], []
    for e, t in enumerate(tris):
        vi, vj = int(t[1]), int(t[2])
        for vk in t:
            vk = int(vk)
            if vi > vj and (vj, vi) in edge_ele:
                ne = edge_ele[(vj, vi)]
                other = [int(w) for w in tris[ne] if w != vi and w != vj][0]
                pairs.append((other, vk))
                ks.append(min(E[e], E[ne]) / (24 * (1 - min(nu[e], nu[ne]) ** 2)) * stiffness)
            vi, vj = vj, vk
    if kind == "angle":
        return len(pairs)
    sv = np.array(pairs, dtype=np.int32).reshape(-1, 2)
    x = np.asarray(state["vx"])
    state["spring_v"] = np.ascontiguousarray(sv)
    state["spring_k"] = np.array(ks, dtype=np.float64)
    state["spring_rl"] = (np.linalg.norm(x[sv[:, 1]] - x[sv[:, 0]], axis=1) if len(sv)
                          else np.zeros(0))
    state["thickness"] = np.float64(thickness)
    return len(pairs)


def cloth_init(mesh, dx: float) -> dict:
    """ToZSCloth (triangles) or ToZSParticles' curve set-up (segments) in FP64:
    the vertex and element arrays of a scenes.ClothMesh."""
    x = np.ascontiguousarray(mesh.x, dtype=np.float32)
    v = None if mesh.v is None else np.ascontiguousarray(mesh.v, dtype=np.float32)
    tris = np.ascontiguousarray(mesh.tris, dtype=np.int32)
    nv, ne = x.shape[0], tris.shape[0]
    state = {k: np.zeros((nv, c) if c > 1 else nv) for k, c in CLOTH_VERT.items()}
    state.update({k: np.zeros((ne, c) if c > 1 else ne) for k, c in CLOTH_ELE.items()})
    state["inds"] = np.zeros((ne, 3), np.int32)
    st = _cloth_struct(mesh, state)
    fn = lib().orc_curve_init_f64 if _is_curve(mesh) else lib().orc_cloth_init_f64
    rc = fn(nv, _ptr(x), _ptr(v), ne, _ptr(tris), float(dx), float(mesh.density), float(mesh.E),
            float(mesh.nu), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle cloth init failed with status {rc}")
    return state


def run_cloth(scene, parts, mesh, state: dict, nsteps: int, dt: float | None = None,
              trackers: np.ndarray | None = None):
    """FP64 substeps of the particles together with one cloth (state from
    cloth_init, copied; mesh None for none) and optional tracker points
    (positions (n, 3)); returns (particles, cloth state, stats), the state
    holding the trackers' "tx", "tv" when given."""
    state = {k: np.array(a, copy=True) for k, a in (state or {}).items()}
    if trackers is not None:
        state["tx"] = np.ascontiguousarray(trackers, dtype=np.float64).reshape(-1, 3).copy()
        state["tv"] = np.zeros_like(state["tx"])
    p = parts.copy(dtype=np.float64)
    for k in ("x", "v", "C", "F", "J", "m", "vol", "mu", "lam", "beta"):
        a = getattr(p, k)
        if a is not None:
            setattr(p, k, np.ascontiguousarray(a, dtype=np.float64))
    p.mat = np.ascontiguousarray(p.mat, dtype=np.int32)
    h = _SceneHolder(scene)
    if mesh is not None:
        h.attach_cloth(_cloth_struct(mesh, state))
    if trackers is not None:
        h.attach_trackers(OrcTrackers(state["tx"].shape[0], state["tx"].ctypes.data,
                                      state["tv"].ctypes.data))
    st = OrcStats()
    rc = lib().orc_run_f64(C.byref(h.s), p.n, _ptr(p.x), _ptr(p.v), _ptr(p.C), _ptr(p.F),
                           _ptr(p.J), _ptr(p.m), _ptr(p.vol), _ptr(p.mat), _ptr(p.mu),
                           _ptr(p.lam), _ptr(p.beta), float(scene.dt if dt is None else dt),
                           int(nsteps), 0, C.byref(st))
    return p, state, {"status": rc, "max_vel_sqr": st.max_vel_sqr, "n_gblocks": st.n_gblocks}


def sym_eig3(A: np.ndarray):
    A = np.ascontiguousarray(A, dtype=np.float64)
    w = np.zeros(3)
    Q = np.zeros(9)
    lib().orc_sym_eig3(_ptr(A), _ptr(w), _ptr(Q))
    return w, Q.reshape(3, 3)


def kirchhoff(material, F: np.ndarray, J: float = 1.0):
    F = np.ascontiguousarray(F, dtype=np.float64)
    tau = np.zeros(9)
    m = make_material(material)
    ok = lib().orc_kirchhoff(C.byref(m), _ptr(F), float(J), _ptr(tau))
    return bool(ok), tau.reshape(3, 3)


def project_dp(material, F: np.ndarray):
    F = np.array(F, dtype=np.float64, copy=True).reshape(9)
    m = make_material(material)
    rc = lib().orc_project_dp(C.byref(m), _ptr(F))
    return rc, F.reshape(3, 3)


def project_hencky(material, F: np.ndarray, logJp: float = 0.0):
    """Von Mises / Cam-Clay return mapping of F: (status, F', log(Jp)')."""
    F = np.array(F, dtype=np.float64, copy=True).reshape(9)
    lj = np.array([logJp], dtype=np.float64)
    m = make_material(material)
    rc = lib().orc_project_hencky(C.byref(m), _ptr(F), _ptr(lj))
    return rc, F.reshape(3, 3), float(lj[0])


def max_threads() -> int:
    return int(lib().orc_max_threads())


def boundary_points_from_mesh(pos: np.ndarray, tris: np.ndarray, dx: float,
                              vel: np.ndarray | None = None) -> dict:
    """ToBoundaryParticles (no sprayed points) in FP64: rows of the mesh's
    vertices, then of its triangles: x, v, m, nrm."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    nv, nt = pos.shape[0], tris.shape[0]
    velp = None
    if vel is not None:
        vel = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3)
        velp = _ptr(vel)
    out = {k: np.zeros((nv + nt, 3) if k != "m" else nv + nt, np.float64)
           for k in ("x", "v", "m", "nrm")}
    rc = lib().orc_boundary_points_from_mesh(nv, _ptr(pos), velp, nt, _ptr(tris), C.c_float(dx),
                                             _ptr(out["x"]), _ptr(out["v"]), _ptr(out["m"]),
                                             _ptr(out["nrm"]))
    if rc != 0:
        raise RuntimeError(f"oracle boundary points failed with status {rc}")
    return out
