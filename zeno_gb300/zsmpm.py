"""Python binding of the zsmpm C ABI (include/zsmpm.h) over ctypes.

This is a thin host-side mirror of the reference's MPM node sequence: a
`Context` is the ZSGrid + ZSPartition + ZSParticles objects of one scene,
and its methods are the nodes (`partition` = ZSPartitionForZSParticles +
ExpandZSPartition, `p2g` = ZSParticleToZSGrid, ...).  Every call goes to the
CUDA library; there is no CPU path.  Loading fails loudly when the library
has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libzsmpm.so")

MPM_OK = 0
STATUS_NAMES = {0: "ok", 1: "invalid", 2: "cuda", 3: "capacity", 4: "out_of_domain", 5: "cfl",
                6: "nan", 7: "timeout", 8: "no_device", 9: "state"}


class MPMError(RuntimeError):
    def __init__(self, code: int, where: str, text: str):
        self.code = code
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)} ({code}): {text}")


class CtxDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("dx", C.c_float), ("block_lo", C.c_int32 * 3),
                ("block_dims", C.c_int32 * 3), ("max_particles", C.c_int64),
                ("max_grid_blocks", C.c_int32), ("flags", C.c_int32)]


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("plasticity", C.c_int32), ("E", C.c_float),
                ("nu", C.c_float), ("density", C.c_float), ("friction_angle_deg", C.c_float),
                ("bulk", C.c_float), ("gamma", C.c_float), ("yield_stress", C.c_float),
                ("cc_beta", C.c_float), ("cc_xi", C.c_float)]


class Boundary(C.Structure):
    _fields_ = [("type", C.c_int32), ("thickness", C.c_int32), ("lo", C.c_int32 * 3),
                ("hi", C.c_int32 * 3)]


class SceneDesc(C.Structure):
    _fields_ = [("dx", C.c_float), ("block_lo", C.c_int32 * 3), ("block_dims", C.c_int32 * 3),
                ("gravity", C.c_float * 3), ("boundary", Boundary)]


class ColliderDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("scene", C.c_int32), ("dims", C.c_int32 * 3),
                ("origin", C.c_float * 3), ("spacing", C.c_float), ("sdf", C.c_void_p),
                ("velocity", C.c_void_p), ("const_velocity", C.c_float * 3),
                ("translation", C.c_float * 3), ("translation_rate", C.c_float * 3),
                ("scale", C.c_float), ("scale_rate", C.c_float), ("ypr_deg", C.c_float * 3)]


class LaunchConfig(C.Structure):
    _fields_ = [("p2g_ctas_per_sm", C.c_int32), ("g2p_ctas_per_sm", C.c_int32),
                ("sort_ctas_per_sm", C.c_int32), ("stream_ctas_per_sm", C.c_int32),
                ("g2p_threads", C.c_int32), ("p2g_shape", C.c_int32),
                ("gather_blocks", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("n_particle_blocks", C.c_int32),
                ("n_grid_blocks", C.c_int32), ("max_vel_sqr", C.c_float), ("status", C.c_int32),
                ("substeps", C.c_int64)]


EXPORTS = ["mpm_abi_version", "mpm_last_error", "mpm_ctx_create", "mpm_ctx_destroy",
           "mpm_batch_create", "mpm_batch_upload",
           "mpm_set_stream", "mpm_set_materials", "mpm_set_boundary", "mpm_set_gravity",
           "mpm_particles_upload", "mpm_particles_upload_async", "mpm_particles_set_lame", "mpm_particles_download", "mpm_partition", "mpm_grid_clear",
           "mpm_p2g", "mpm_grid_update", "mpm_apply_boundary", "mpm_apply_walls",
           "mpm_apply_collider", "mpm_set_transfer", "mpm_compute_particle_beta",
           "mpm_particles_get_attr", "mpm_particles_set_attr", "mpm_compute_von_mises",
           "mpm_frame_begin", "mpm_frame_wait", "mpm_cloth_create", "mpm_cloth_download",
           "mpm_cloth_upload", "mpm_checkpoint_write", "mpm_checkpoint_read",
           "mpm_cloth_add_bending",
           "mpm_trackers_create", "mpm_trackers_download",
           "mpm_g2p", "mpm_return_mapping",
           "mpm_substep", "mpm_substep_timed", "mpm_sync", "mpm_get_stats", "mpm_partition_download",
           "mpm_grid_download", "mpm_partition_noalloc", "mpm_set_launch_config",
           "mpm_get_launch_config", "mpm_set_differentiable", "mpm_state_save",
           "mpm_state_load", "mpm_adjoint_substep", "mpm_rollout_forward", "mpm_rollout_backward", "mpm_snapshot_floats", "mpm_add_collider", "mpm_clear_colliders",
           "mpm_step_colliders", "mpm_set_auto_regrow", "mpm_get_domain",
           "mpm_set_persistent", "mpm_barrier_selftest", "mpm_set_grid_boundary",
           "mpm_clear_grid_boundary", "mpm_apply_grid_boundary", "mpm_boundary_points_from_mesh"]

STAGES = ["bin", "scan", "scatter", "sort", "p2g", "grid_update", "g2p"]
# differentiable form (include/zsmpm.h): state planes x 3, v 3, C 9, F 9, J,
# m, vol, mu, lam, material id, upload index; adjoint planes x v C F J
STATE_PLANES = 31
ADJ_PLANES = 25

_lib = None


def load(path: str = LIB_PATH):
    """Load libzsmpm.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    P = C.c_void_p
    i32, i64, f32 = C.c_int32, C.c_int64, C.c_float
    sig = {
        "mpm_abi_version": ([], i32),
        "mpm_last_error": ([], C.c_char_p),
        "mpm_ctx_create": ([C.POINTER(CtxDesc), C.POINTER(C.c_void_p)], i32),
        "mpm_ctx_destroy": ([P], i32),
        "mpm_batch_create": ([i32, C.POINTER(SceneDesc), i32, i64, i32, C.POINTER(C.c_void_p)],
                             i32),
        "mpm_batch_upload": ([P, P, i64] + [P] * 10, i32),
        "mpm_set_stream": ([P, P], i32),
        "mpm_set_materials": ([P, C.POINTER(Material), i32], i32),
        "mpm_set_boundary": ([P, C.POINTER(Boundary)], i32),
        "mpm_set_gravity": ([P, f32, f32, f32], i32),
        "mpm_add_collider": ([P, P, P], i32),
        "mpm_clear_colliders": ([P], i32),
        "mpm_step_colliders": ([P, i32, f32], i32),
        "mpm_particles_upload": ([P, i64] + [P] * 10, i32),
        "mpm_particles_upload_async": ([P, i64] + [P] * 10, i32),
        "mpm_particles_set_lame": ([P, P, P], i32),
        "mpm_particles_download": ([P] + [P] * 5, i32),
        "mpm_partition": ([P], i32),
        "mpm_grid_clear": ([P], i32),
        "mpm_p2g": ([P, f32], i32),
        "mpm_grid_update": ([P, f32, P], i32),
        "mpm_apply_boundary": ([P], i32),
        "mpm_apply_walls": ([P], i32),
        "mpm_set_transfer": ([P, i32], i32),
        "mpm_compute_particle_beta": ([P, f32, i32], i32),
        "mpm_particles_get_attr": ([P, C.c_char_p, P], i32),
        "mpm_particles_set_attr": ([P, C.c_char_p, P], i32),
        "mpm_compute_von_mises": ([P, i32], i32),
        "mpm_cloth_create": ([P, P], i32),
        "mpm_trackers_create": ([P, i64, P, P], i32),
        "mpm_cloth_add_bending": ([P, i32, C.c_float, C.c_float, P], i32),
        "mpm_trackers_download": ([P, P, P], i32),
        "mpm_cloth_download": ([P] + [P] * 8, i32),
        "mpm_cloth_upload": ([P] + [P] * 8, i32),
        "mpm_checkpoint_write": ([P, C.c_char_p], i32),
        "mpm_checkpoint_read": ([P, C.c_char_p], i32),
        "mpm_frame_begin": ([P, P, P], i32),
        "mpm_frame_wait": ([P], i32),
        "mpm_apply_collider": ([P, i32], i32),
        "mpm_g2p": ([P, f32], i32),
        "mpm_return_mapping": ([P], i32),
        "mpm_substep": ([P, f32, i32], i32),
        "mpm_substep_timed": ([P, f32, P, i32], i32),
        "mpm_sync": ([P], i32),
        "mpm_get_stats": ([P, C.POINTER(Stats)], i32),
        "mpm_partition_download": ([P, P, P, P, i64, P, P, P, i64], i32),
        "mpm_grid_download": ([P, P, i64], i32),
        "mpm_partition_noalloc": ([P, i64, f32, P, P, P, P, P, i64, P, P], i32),
        "mpm_set_launch_config": ([P, C.POINTER(LaunchConfig)], i32),
        "mpm_get_launch_config": ([P, C.POINTER(LaunchConfig)], i32),
        "mpm_set_differentiable": ([P, i32], i32),
        "mpm_rollout_forward": ([P, f32, i32, i32, P, P, P, P], i32),
        "mpm_snapshot_floats": ([P, P], i32),
        "mpm_rollout_backward": ([P, f32, i32, i32, P, P, P, P, P, P], i32),
        "mpm_set_auto_regrow": ([P, i32], i32),
        "mpm_get_domain": ([P, P, P, P], i32),
        "mpm_set_persistent": ([P, i32, C.c_uint64], i32),
        "mpm_set_grid_boundary": ([P, i32, C.c_int64, C.c_int64, P, P, P, P], i32),
        "mpm_clear_grid_boundary": ([P], i32),
        "mpm_apply_grid_boundary": ([P], i32),
        "mpm_boundary_points_from_mesh": ([C.c_int64, P, P, C.c_int64, P, f32, P, P, P, P], i32),
        "mpm_barrier_selftest": ([P, C.c_uint64, P], i32),
        "mpm_state_save": ([P, P], i32),
        "mpm_state_load": ([P, P], i32),
        "mpm_adjoint_substep": ([P, f32, P, P, P, P], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a, shape):
    if a is None:
        return None
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(shape))


class ClothDesc(C.Structure):
    _fields_ = [("n_verts", C.c_int64), ("x", C.c_void_p), ("v", C.c_void_p),
                ("n_tris", C.c_int64), ("tris", C.c_void_p), ("model", C.c_int32),
                ("E", C.c_float), ("nu", C.c_float), ("density", C.c_float),
                ("stiffness_shear", C.c_float), ("stiffness_normal", C.c_float),
                ("friction_angle", C.c_float), ("damping_coeff", C.c_float),
                ("kind", C.c_int32)]


def boundary_points_from_mesh(pos, tris, dx: float, vel=None) -> dict:
    """ToBoundaryParticles (host code of the library, no GPU): rows of the
    mesh's vertices, then one per triangle: x, v, m, nrm (float32)."""
    L = load()
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    nv, nt = pos.shape[0], tris.shape[0]
    if vel is not None:
        vel = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3)
    out = {k: np.zeros((nv + nt, 3) if k != "m" else nv + nt, np.float32)
           for k in ("x", "v", "m", "nrm")}
    rc = L.mpm_boundary_points_from_mesh(nv, _p(pos), _p(vel) if vel is not None else None, nt,
                                         _p(tris), float(dx), _p(out["x"]), _p(out["v"]),
                                         _p(out["m"]), _p(out["nrm"]))
    if rc != 0:
        raise MPMError(rc, "mpm_boundary_points_from_mesh", L.mpm_last_error().decode())
    return out


def mesh_grid_boundary(pos, tris, dx: float, type: int, vel=None):
    """A scenes.GridBoundary of a triangle mesh (ToBoundaryParticles)."""
    from .scenes import GridBoundary
    o = boundary_points_from_mesh(pos, tris, dx, vel)
    return GridBoundary(type=int(type), x=o["x"], v=o["v"], m=o["m"], nrm=o["nrm"],
                        n_verts=int(np.asarray(pos).reshape(-1, 3).shape[0]))


class Context:
    """One MPM scene on one GPU (ZSGrid + ZSPartition + ZSParticles)."""

    def __init__(self, scene, max_particles: int, device: int = 0, max_grid_blocks: int = 0):
        L = load()
        self._L = L
        desc = CtxDesc(device, float(scene.dx), (C.c_int32 * 3)(*scene.block_lo),
                       (C.c_int32 * 3)(*scene.block_dims), int(max_particles),
                       int(max_grid_blocks), 0)
        h = C.c_void_p()
        self._check(L.mpm_ctx_create(C.byref(desc), C.byref(h)), "mpm_ctx_create")
        self.h = h
        self.scene = scene
        self.n = 0
        self.set_materials(scene.materials)
        self.set_boundary(scene.bc_type, scene.bc_thickness, scene.bc_lo, scene.bc_hi)
        self.set_gravity(*scene.gravity)
        for c in getattr(scene, "colliders", []) or []:
            self.add_collider(c)
        if getattr(scene, "transfer", 0):
            self.set_transfer(scene.transfer)
        if getattr(scene, "grid_boundary", None) is not None:
            self.set_grid_boundary(scene.grid_boundary)

    def set_transfer(self, scheme: int):
        """MakeZSGrid "transfer": scenes.TRANSFER_APIC / FLIP / AFLIP."""
        self._check(self._L.mpm_set_transfer(self.h, int(scheme)), "mpm_set_transfer")

    def compute_particle_beta(self, dt: float, collider: int = -1):
        """ComputeParticleBeta: the volume criterion, and with a collider id
        first the level-set test of that collider."""
        self._check(self._L.mpm_compute_particle_beta(self.h, float(dt), int(collider)),
                    "mpm_compute_particle_beta")

    def get_attr(self, name: str) -> np.ndarray:
        out = np.empty(self.n, np.float32)
        self._check(self._L.mpm_particles_get_attr(self.h, name.encode(), _p(out)),
                    "mpm_particles_get_attr")
        return out

    def set_attr(self, name: str, values):
        vals = _f32(values, (self.n,))
        self._check(self._L.mpm_particles_set_attr(self.h, name.encode(), _p(vals)),
                    "mpm_particles_set_attr")

    def add_cloth(self, mesh):
        """ToZSCloth for a scenes.ClothMesh of triangles, or ToZSParticles'
        curve set-up for one of segments (tris of shape (n, 2)): the mesh is
        stepped with the particles by every substep entry point."""
        x = np.ascontiguousarray(mesh.x, dtype=np.float32)
        v = None if mesh.v is None else np.ascontiguousarray(mesh.v, dtype=np.float32)
        tris = np.ascontiguousarray(mesh.tris, dtype=np.int32)
        desc = ClothDesc(x.shape[0], x.ctypes.data, v.ctypes.data if v is not None else None,
                         tris.shape[0], tris.ctypes.data, int(mesh.model), float(mesh.E),
                         float(mesh.nu), float(mesh.density), float(mesh.gamma), float(mesh.k),
                         float(mesh.fa), float(mesh.dc), 1 if tris.shape[1] == 2 else 0)
        self._check(self._L.mpm_cloth_create(self.h, C.byref(desc)), "mpm_cloth_create")
        self._cloth_n = (x.shape[0], tris.shape[0])

    def add_cloth_bending(self, stiffness: float, kind: str = "vertex", thickness: float = None) -> int:
        """ConstructBendingSprings on the context's cloth ("vertex" or "angle";
        thickness defaults to the grid dx); returns the pair / hinge count."""
        t = {"vertex": 0, "element": 1, "angle": 2}[kind]
        n = C.c_int64(0)
        th = self.scene.dx if thickness is None else thickness
        self._check(self._L.mpm_cloth_add_bending(self.h, t, float(stiffness), float(th),
                                                  C.byref(n)), "mpm_cloth_add_bending")
        return int(n.value)

    def cloth_beta(self) -> np.ndarray:
        """The cloth vertices' beta (ComputeParticleBeta on the cloth)."""
        out = np.empty(self._cloth_n[0], np.float32)
        self._check(self._L.mpm_particles_get_attr(self.h, b"cloth_beta", _p(out)),
                    "mpm_particles_get_attr")
        return out

    def set_cloth_beta(self, values):
        vals = _f32(values, (self._cloth_n[0],))
        self._check(self._L.mpm_particles_set_attr(self.h, b"cloth_beta", _p(vals)),
                    "mpm_particles_set_attr")

    def add_trackers(self, x, v=None):
        """ToTrackerParticles: points advected by the grid in every substep."""
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 3)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float32).reshape(-1, 3)
        self._check(self._L.mpm_trackers_create(self.h, x.shape[0], _p(x), _p(v)),
                    "mpm_trackers_create")
        self._n_trackers = x.shape[0]

    def trackers_download(self):
        x = np.empty((self._n_trackers, 3), np.float32)
        v = np.empty_like(x)
        self._check(self._L.mpm_trackers_download(self.h, _p(x), _p(v)), "mpm_trackers_download")
        return x, v

    def cloth_download(self) -> dict:
        nv, ne = self._cloth_n
        out = {"vx": np.empty((nv, 3), np.float32), "vv": np.empty((nv, 3), np.float32),
               "vC": np.empty((nv, 9), np.float32), "ex": np.empty((ne, 3), np.float32),
               "ev": np.empty((ne, 3), np.float32), "eC": np.empty((ne, 9), np.float32),
               "eF": np.empty((ne, 9), np.float32), "ed": np.empty((ne, 9), np.float32)}
        self._check(self._L.mpm_cloth_download(self.h, *[_p(out[k]) for k in
                                                         ("vx", "vv", "vC", "ex", "ev", "eC",
                                                          "eF", "ed")]), "mpm_cloth_download")
        return out

    def checkpoint_write(self, path: str):
        """The solver state to a file (mpm_checkpoint_write)."""
        self._check(self._L.mpm_checkpoint_write(self.h, os.fsencode(path)),
                    "mpm_checkpoint_write")

    def checkpoint_read(self, path: str):
        """The solver state from a file of a context with the same scene."""
        self._check(self._L.mpm_checkpoint_read(self.h, os.fsencode(path)), "mpm_checkpoint_read")
        self.n = self.stats()["n_particles"]  # the checkpoint's particles

    def cloth_upload(self, state: dict):
        """The inverse of cloth_download: arrays given by key (vx, vv, vC,
        ex, ev, eC, eF, ed) replace the cloth's, the others stay."""
        nv, ne = self._cloth_n
        shapes = {"vx": (nv, 3), "vv": (nv, 3), "vC": (nv, 9), "ex": (ne, 3), "ev": (ne, 3),
                  "eC": (ne, 9), "eF": (ne, 9), "ed": (ne, 9)}
        arrs = [None if state.get(k) is None else _f32(state[k], shapes[k]) for k in shapes]
        self._check(self._L.mpm_cloth_upload(self.h, *[_p(a) for a in arrs]), "mpm_cloth_upload")

    def compute_von_mises(self, by_log1p: bool = True):
        """ComputeVonMises; the result is the attribute "vms"."""
        self._check(self._L.mpm_compute_von_mises(self.h, 1 if by_log1p else 0),
                    "mpm_compute_von_mises")

    def frame_begin(self, x, v):
        """Asynchronous write-back of x, v (caller-owned float32 (n, 3) arrays,
        page-locked for an overlapped copy); frame_wait() before reading."""
        self._frame = (x, v)
        self._check(self._L.mpm_frame_begin(self.h, _p(x), _p(v)), "mpm_frame_begin")

    def frame_wait(self):
        self._check(self._L.mpm_frame_wait(self.h), "mpm_frame_wait")

    def add_collider(self, c, scene: int = None) -> int:
        """mpm_add_collider for a scenes.Collider; returns its index."""
        sdf = np.ascontiguousarray(c.sdf, dtype=np.float32)
        nz, ny, nx = sdf.shape
        vel = None if c.velocity is None else np.ascontiguousarray(c.velocity, dtype=np.float32)
        if vel is not None and vel.shape != (3, nz, ny, nx):
            raise ValueError("collider velocity must have shape (3,) + sdf.shape")
        desc = ColliderDesc(int(c.type), int(c.scene if scene is None else scene),
                            (C.c_int32 * 3)(nx, ny, nz), (C.c_float * 3)(*c.origin),
                            float(c.spacing), sdf.ctypes.data,
                            vel.ctypes.data if vel is not None else None,
                            (C.c_float * 3)(*c.const_velocity), (C.c_float * 3)(*c.translation),
                            (C.c_float * 3)(*c.translation_rate), float(c.scale),
                            float(c.scale_rate), (C.c_float * 3)(*c.ypr_deg))
        idx = C.c_int32(-1)
        self._check(self._L.mpm_add_collider(self.h, C.byref(desc), C.byref(idx)),
                    "mpm_add_collider")
        return idx.value

    def clear_colliders(self):
        self._check(self._L.mpm_clear_colliders(self.h), "mpm_clear_colliders")

    def set_grid_boundary(self, gb):
        """mpm_set_grid_boundary for a scenes.GridBoundary."""
        f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
        x, v, m, nrm = f(gb.x), f(gb.v), f(gb.m), f(gb.nrm)
        n = m.shape[0]
        self._check(self._L.mpm_set_grid_boundary(self.h, int(gb.type), int(gb.n_verts),
                                                  int(n - gb.n_verts), _p(x), _p(v), _p(m),
                                                  _p(nrm)), "mpm_set_grid_boundary")

    def clear_grid_boundary(self):
        self._check(self._L.mpm_clear_grid_boundary(self.h), "mpm_clear_grid_boundary")

    def apply_grid_boundary(self):
        self._check(self._L.mpm_apply_grid_boundary(self.h), "mpm_apply_grid_boundary")

    def step_colliders(self, dt: float, collider: int = -1):
        """StepZSBoundary: b += db/dt dt, s += ds/dt dt (stage path), for one
        collider or (-1) every collider."""
        self._check(self._L.mpm_step_colliders(self.h, int(collider), float(dt)),
                    "mpm_step_colliders")

    @property
    def dir_size(self) -> int:
        _, dims, _ = self.domain()  # the directory may have grown
        return int(np.prod(dims))

    def _check(self, rc: int, where: str):
        if rc != MPM_OK:
            raise MPMError(rc, where, self._L.mpm_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self._L.mpm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ConfigConstitutiveModel / ToZSBoundary / UpdateZSGrid inputs
    def set_materials(self, mats):
        arr = (Material * len(mats))(*[Material(int(m.type), int(m.plasticity), float(m.E),
                                                float(m.nu), float(m.density),
                                                float(m.friction_angle_deg), float(m.bulk),
                                                float(m.gamma),
                                                float(getattr(m, "yield_stress", 1e5)),
                                                float(getattr(m, "cc_beta", 2.0)),
                                                float(getattr(m, "cc_xi", 1.0)))
                                       for m in mats])
        self._check(self._L.mpm_set_materials(self.h, arr, len(mats)), "mpm_set_materials")

    def set_boundary(self, bc_type, thickness, lo, hi):
        b = Boundary(int(bc_type), int(thickness), (C.c_int32 * 3)(*lo), (C.c_int32 * 3)(*hi))
        self._check(self._L.mpm_set_boundary(self.h, C.byref(b)), "mpm_set_boundary")

    def set_gravity(self, gx, gy, gz):
        self._check(self._L.mpm_set_gravity(self.h, gx, gy, gz), "mpm_set_gravity")

    def set_stream(self, stream_ptr: int | None):
        self._check(self._L.mpm_set_stream(self.h, C.c_void_p(stream_ptr or 0)), "mpm_set_stream")

    # ToZSParticles / UpdatePrimitiveFromZSParticles
    def upload(self, parts):
        n = parts.n
        x = _f32(parts.x, (n, 3))
        v = _f32(parts.v, (n, 3))
        Cm = _f32(parts.C, (n, 9))
        F = _f32(parts.F, (n, 9))
        J = _f32(parts.J, (n,))
        m = _f32(parts.m, (n,))
        vol = _f32(parts.vol, (n,))
        mat = np.ascontiguousarray(parts.mat, dtype=np.int32)
        mu = _f32(parts.mu, (n,))
        lam = _f32(parts.lam, (n,))
        self._keep = (x, v, Cm, F, J, m, vol, mat, mu, lam)
        self._check(self._L.mpm_particles_upload(self.h, n, _p(x), _p(v), _p(Cm), _p(F), _p(J),
                                                 _p(m), _p(vol), _p(mat), _p(mu), _p(lam)),
                    "mpm_particles_upload")
        self.n = n
        if getattr(parts, "beta", None) is not None:
            self.set_attr("beta", parts.beta)

    def upload_async(self, parts):
        """mpm_particles_upload_async: returns once the copies and the
        conversion are enqueued; the arrays (kept referenced here) must stay
        unchanged until the next sync, and page-locked arrays keep the copies
        asynchronous.  A bad material id surfaces at the next sync."""
        n = parts.n
        x = _f32(parts.x, (n, 3))
        v = _f32(parts.v, (n, 3))
        Cm = _f32(parts.C, (n, 9))
        F = _f32(parts.F, (n, 9))
        J = _f32(parts.J, (n,))
        m = _f32(parts.m, (n,))
        vol = _f32(parts.vol, (n,))
        mat = np.ascontiguousarray(parts.mat, dtype=np.int32)
        mu = _f32(parts.mu, (n,))
        lam = _f32(parts.lam, (n,))
        self._keep = (x, v, Cm, F, J, m, vol, mat, mu, lam)
        self._check(self._L.mpm_particles_upload_async(self.h, n, _p(x), _p(v), _p(Cm), _p(F),
                                                       _p(J), _p(m), _p(vol), _p(mat), _p(mu),
                                                       _p(lam)),
                    "mpm_particles_upload_async")
        self.n = n

    def upload_raw(self, n, x, v=None, Cm=None, F=None, J=None, m=None, vol=None, mat=None,
                   mu=None, lam=None):
        """Upload from caller-owned contiguous float32 / int32 arrays (no copy)."""
        self._check(self._L.mpm_particles_upload(self.h, n, _p(x), _p(v), _p(Cm), _p(F), _p(J),
                                                 _p(m), _p(vol), _p(mat), _p(mu), _p(lam)),
                    "mpm_particles_upload")
        self.n = n

    def set_lame(self, mu, lam):
        """AdjustParticleMaterial: per-particle mu / lam in upload order."""
        mu = _f32(mu, (self.n,))
        lam = _f32(lam, (self.n,))
        self._check(self._L.mpm_particles_set_lame(self.h, _p(mu), _p(lam)),
                    "mpm_particles_set_lame")

    def download(self, channels=("x", "v", "C", "F", "J")) -> dict:
        n = self.n
        out = {}
        shapes = {"x": (n, 3), "v": (n, 3), "C": (n, 3, 3), "F": (n, 3, 3), "J": (n,)}
        for k in ("x", "v", "C", "F", "J"):
            out[k] = np.empty(shapes[k], np.float32) if k in channels else None
        self._check(self._L.mpm_particles_download(self.h, _p(out["x"]), _p(out["v"]),
                                                   _p(out["C"]), _p(out["F"]), _p(out["J"])),
                    "mpm_particles_download")
        return {k: v for k, v in out.items() if v is not None}

    def download_raw(self, x=None, v=None):
        self._check(self._L.mpm_particles_download(self.h, _p(x), _p(v), None, None, None),
                    "mpm_particles_download")

    # the substep nodes
    def partition(self):
        self._check(self._L.mpm_partition(self.h), "mpm_partition")

    def grid_clear(self):
        self._check(self._L.mpm_grid_clear(self.h), "mpm_grid_clear")

    def p2g(self, dt):
        self._check(self._L.mpm_p2g(self.h, dt), "mpm_p2g")

    def grid_update(self, dt, read_max: bool = True):
        out = C.c_float(0.0)
        self._check(self._L.mpm_grid_update(self.h, dt, C.byref(out) if read_max else None),
                    "mpm_grid_update")
        return out.value if read_max else None

    def apply_boundary(self):
        self._check(self._L.mpm_apply_boundary(self.h), "mpm_apply_boundary")

    def apply_walls(self):
        self._check(self._L.mpm_apply_walls(self.h), "mpm_apply_walls")

    def apply_collider(self, collider=-1):
        self._check(self._L.mpm_apply_collider(self.h, collider), "mpm_apply_collider")

    def g2p(self, dt):
        self._check(self._L.mpm_g2p(self.h, dt), "mpm_g2p")

    def return_mapping(self):
        self._check(self._L.mpm_return_mapping(self.h), "mpm_return_mapping")

    def staged_substep(self, dt):
        """One substep through the node-by-node entry points."""
        self.partition()
        self.grid_clear()
        self.p2g(dt)
        vmax = self.grid_update(dt, read_max=False)
        self.apply_boundary()
        self.g2p(dt)
        self.return_mapping()
        return vmax

    def substep(self, dt, n: int = 1):
        self._check(self._L.mpm_substep(self.h, dt, int(n)), "mpm_substep")

    def substep_timed(self, dt) -> dict:
        """One substep with CUDA events between stages: device ms per stage."""
        ms = np.zeros(len(STAGES), np.float32)
        self._check(self._L.mpm_substep_timed(self.h, dt, _p(ms), len(STAGES)),
                    "mpm_substep_timed")
        return dict(zip(STAGES, ms.tolist()))

    def sync(self):
        self._check(self._L.mpm_sync(self.h), "mpm_sync")

    # growing directory
    def set_auto_regrow(self, on: bool = True):
        self._check(self._L.mpm_set_auto_regrow(self.h, 1 if on else 0), "mpm_set_auto_regrow")

    # one persistent kernel per substep (include/zsmpm.h: mpm_set_persistent)
    BARRIER_LIMIT_DEFAULT = 1 << 24

    def set_persistent(self, on: bool = True, barrier_limit: int = BARRIER_LIMIT_DEFAULT):
        self._check(self._L.mpm_set_persistent(self.h, 1 if on else 0, int(barrier_limit)),
                    "mpm_set_persistent")

    def barrier_selftest(self, barrier_limit: int = 1000) -> bool:
        """True when waits at a barrier nothing completes gave up and said so."""
        t = C.c_int32(0)
        self._check(self._L.mpm_barrier_selftest(self.h, int(barrier_limit), C.byref(t)),
                    "mpm_barrier_selftest")
        return bool(t.value)

    def domain(self):
        """(block_lo, block_dims, n_regrows) of the directory."""
        lo = (C.c_int32 * 3)()
        dims = (C.c_int32 * 3)()
        nr = C.c_int32(0)
        self._check(self._L.mpm_get_domain(self.h, lo, dims, C.byref(nr)), "mpm_get_domain")
        return tuple(lo), tuple(dims), nr.value

    # differentiable form: device pointers (ints); a state is STATE_PLANES
    # planes of n floats in the store's slot order, an adjoint ADJ_PLANES
    def set_differentiable(self, on: bool = True):
        self._check(self._L.mpm_set_differentiable(self.h, 1 if on else 0),
                    "mpm_set_differentiable")

    def snapshot_floats(self) -> int:
        v = C.c_int64(0)
        self._check(self._L.mpm_snapshot_floats(self.h, C.byref(v)), "mpm_snapshot_floats")
        return v.value

    def rollout_forward(self, dt, n_substeps: int, every: int, state0: int, ckpts: int,
                        final: int, seg_states: int = 0):
        """seg_states (0: none): the backward's scratch, which then receives
        the last segment's states so that the backward skips recomputing it."""
        self._check(self._L.mpm_rollout_forward(self.h, dt, int(n_substeps), int(every),
                                                C.c_void_p(state0), C.c_void_p(ckpts),
                                                C.c_void_p(seg_states or None),
                                                C.c_void_p(final)), "mpm_rollout_forward")

    def rollout_backward(self, dt, n_substeps: int, every: int, ckpts: int, seg_states: int,
                         adj: int, adj_tmp: int, grad_mu: int, grad_lam: int):
        self._check(self._L.mpm_rollout_backward(
            self.h, dt, int(n_substeps), int(every), C.c_void_p(ckpts), C.c_void_p(seg_states),
            C.c_void_p(adj), C.c_void_p(adj_tmp), C.c_void_p(grad_mu), C.c_void_p(grad_lam)),
            "mpm_rollout_backward")

    def state_save(self, dst_ptr: int):
        self._check(self._L.mpm_state_save(self.h, C.c_void_p(dst_ptr)), "mpm_state_save")

    def state_load(self, src_ptr: int):
        self._check(self._L.mpm_state_load(self.h, C.c_void_p(src_ptr)), "mpm_state_load")

    def adjoint_substep(self, dt, adj_next: int, adj_prev: int, grad_mu: int, grad_lam: int):
        self._check(self._L.mpm_adjoint_substep(self.h, dt, C.c_void_p(adj_next),
                                                C.c_void_p(adj_prev), C.c_void_p(grad_mu),
                                                C.c_void_p(grad_lam)), "mpm_adjoint_substep")

    def set_launch_config(self, cfg: dict):
        lc = LaunchConfig(*(int(cfg.get(k, 0)) for k, _ in LaunchConfig._fields_))
        self._check(self._L.mpm_set_launch_config(self.h, C.byref(lc)), "mpm_set_launch_config")

    def get_launch_config(self) -> dict:
        lc = LaunchConfig()
        self._check(self._L.mpm_get_launch_config(self.h, C.byref(lc)), "mpm_get_launch_config")
        return {k: getattr(lc, k) for k, _ in LaunchConfig._fields_}

    def stats(self) -> dict:
        s = Stats()
        self._check(self._L.mpm_get_stats(self.h, C.byref(s)), "mpm_get_stats")
        return {"n_particles": s.n_particles, "n_particle_blocks": s.n_particle_blocks,
                "n_grid_blocks": s.n_grid_blocks, "max_vel_sqr": s.max_vel_sqr,
                "status": s.status, "substeps": s.substeps}

    def partition_download(self) -> dict:
        D = self.dir_size
        n_pb = np.zeros(1, np.int32)
        n_gb = np.zeros(1, np.int32)
        pb_dir = np.zeros(D, np.int32)
        pb_count = np.zeros(D, np.int32)
        gb_dir = np.zeros(D, np.int32)
        perm = np.zeros(max(self.n, 1), np.int32)
        self._check(self._L.mpm_partition_download(self.h, _p(n_pb), _p(pb_dir), _p(pb_count), D,
                                                   _p(perm), _p(n_gb), _p(gb_dir), D),
                    "mpm_partition_download")
        return {"pb_dir": pb_dir[:n_pb[0]].copy(), "pb_count": pb_count[:n_pb[0]].copy(),
                "perm": perm[:self.n].astype(np.int64), "gb_dir": gb_dir[:n_gb[0]].copy()}

    def grid_download(self) -> np.ndarray:
        st = self.stats()
        ng = st["n_grid_blocks"]
        out = np.zeros((max(ng, 1), 64, 4), np.float32)
        self._check(self._L.mpm_grid_download(self.h, _p(out), out.size), "mpm_grid_download")
        return out[:ng]


class BatchContext(Context):
    """Many independent scenes in one context: every stage of a substep is one
    persistent launch over the blocks of all scenes.  Materials of all scenes
    share one table; each particle carries its material id."""

    def __init__(self, scenes, materials, max_particles: int, device: int = 0,
                 max_grid_blocks: int = 0):
        L = load()
        self._L = L
        arr = (SceneDesc * len(scenes))(*[
            SceneDesc(float(sc.dx), (C.c_int32 * 3)(*sc.block_lo),
                      (C.c_int32 * 3)(*sc.block_dims), (C.c_float * 3)(*sc.gravity),
                      Boundary(int(sc.bc_type), int(sc.bc_thickness),
                               (C.c_int32 * 3)(*sc.bc_lo), (C.c_int32 * 3)(*sc.bc_hi)))
            for sc in scenes])
        h = C.c_void_p()
        self._check(L.mpm_batch_create(device, arr, len(scenes), int(max_particles),
                                       int(max_grid_blocks), C.byref(h)), "mpm_batch_create")
        self.h = h
        self.scenes = scenes
        self.scene = scenes[0]
        self.n = 0
        self.set_materials(materials)

    @property
    def dir_size(self) -> int:
        return int(sum(int(np.prod(sc.block_dims)) for sc in self.scenes))

    def upload_batch(self, parts, offsets):
        n = parts.n
        offs = np.ascontiguousarray(offsets, dtype=np.int64)
        x = _f32(parts.x, (n, 3))
        v = _f32(parts.v, (n, 3))
        Cm = _f32(parts.C, (n, 9))
        F = _f32(parts.F, (n, 9))
        J = _f32(parts.J, (n,))
        m = _f32(parts.m, (n,))
        vol = _f32(parts.vol, (n,))
        mat = np.ascontiguousarray(parts.mat, dtype=np.int32)
        mu = _f32(parts.mu, (n,))
        lam = _f32(parts.lam, (n,))
        self._keep = (offs, x, v, Cm, F, J, m, vol, mat, mu, lam)
        self._check(self._L.mpm_batch_upload(self.h, _p(offs), n, _p(x), _p(v), _p(Cm), _p(F),
                                             _p(J), _p(m), _p(vol), _p(mat), _p(mu), _p(lam)),
                    "mpm_batch_upload")
        self.n = n


def concat_scenes(pairs):
    """(scene, particles) pairs -> (scenes, shared material table, particles
    with remapped material ids, scene offsets)."""
    from . import scenes as S
    mats, scenes_out, chunks, offsets = [], [], [], [0]
    for scene, p in pairs:
        ids = []
        for m in scene.materials:  # identical materials share one table entry
            if m not in mats:
                mats.append(m)
            ids.append(mats.index(m))
        scenes_out.append(scene)
        q = p.copy()
        q.mat = np.asarray(ids, dtype=np.int32)[q.mat] if q.n else q.mat.astype(np.int32)
        chunks.append(q)
        offsets.append(offsets[-1] + q.n)

    def cat(k):
        arrs = [getattr(c, k) for c in chunks]
        if any(a is None for a in arrs):
            return None
        return np.concatenate(arrs)
    parts = S.Particles(*(cat(k) for k in ("x", "v", "C", "F", "J", "m", "vol", "mat", "mu",
                                            "lam")))
    return scenes_out, mats, parts, np.array(offsets, dtype=np.int64)


# ---------------------------------------------------------------------------
# the C++ node layer (libzsmpm_nodes.so): zeno's MPM nodes over this ABI

NODES_LIB_PATH = os.path.join(PKG, "libzsmpm_nodes.so")
_nodes = None


def load_nodes(path: str = NODES_LIB_PATH):
    global _nodes
    if _nodes is not None:
        return _nodes
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    L.zsn_descriptors_json.argtypes = [C.c_char_p, C.c_int64]
    L.zsn_descriptors_json.restype = C.c_int32
    P = C.c_void_p
    L.zsn_run_graph.argtypes = [C.c_int32, C.c_int64, P, P, C.c_float, C.c_char_p, C.c_char_p,
                                C.c_float, C.c_float, C.c_float, C.c_float, C.c_char_p,
                                C.c_int32, C.c_float, C.c_float, C.c_int32, P, P, P,
                                C.c_char_p, C.c_int64, C.c_char_p, P, C.c_char_p, C.c_char_p,
                                C.c_int64, P, P, C.c_int64, P, P, P, P, C.c_int64, P, P, P,
                                C.c_char_p, C.c_char_p, C.c_float, C.c_char_p, C.c_int32, P,
                                C.c_char_p, C.c_int64, P, P, C.c_int64, P, C.c_char_p,
                                C.c_int64, P]
    L.zsn_run_graph.restype = C.c_int32
    L.zsn_config_model.argtypes = [C.c_float, C.c_float, C.c_float, C.c_char_p, C.c_char_p,
                                   C.c_char_p, C.c_float, C.c_float, C.c_char_p,
                                   C.POINTER(Material), P, C.c_char_p, C.c_int64]
    L.zsn_config_model.restype = C.c_int32
    _nodes = L
    return L


def node_descriptors() -> dict:
    import json
    L = load_nodes()
    n = L.zsn_descriptors_json(None, 0)
    cap = 1 << 16
    while True:
        buf = C.create_string_buffer(cap)
        n = L.zsn_descriptors_json(buf, cap)
        if n < cap:
            return json.loads(buf.value.decode())
        cap = 2 * n


def config_model(type="fcr", plasticity="none", aniso="none", E=1e4, nu=0.4, dx=0.1, ppc=8.0,
                 density=1000.0, params=None):
    """Apply one ConfigConstitutiveModel node (params: its "params" dict,
    {key: number}); returns (mpm_material fields as a dict, particle volume).
    Runs on the host only: the node makes no device call."""
    L = load_nodes()
    mat = Material()
    vol = np.zeros(1, np.float32)
    err = C.create_string_buffer(1024)
    ptxt = ";".join(f"{k}={float(v)!r}" for k, v in (params or {}).items()).encode()
    rc = L.zsn_config_model(dx, ppc, density, type.encode(), aniso.encode(), plasticity.encode(),
                            E, nu, ptxt, C.byref(mat), _p(vol), err, 1024)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return {k: getattr(mat, k) for k, _ in Material._fields_}, float(vol[0])


def run_node_graph(x, v, dx, type="fcr", plasticity="none", E=1e4, nu=0.4, density=1000.0,
                   ppc=8.0, bc="sticky", thickness=3, dt=1e-4, gravity=-9.8, substeps=1,
                   fused=False, levelset=None, transfer="apic", cloth=None, trackers=None,
                   write_path=None, bending=None, attr=None, params=None, boundary_mesh=None,
                   tracker_tets=None):
    """Run the zeno MPM substep graph headless through the C++ node layer.
    levelset: optional dict for a MakeZSLevelSet -> ToZSBoundary collider
    applied after the walls -- in the stage graph through StepZSBoundary and a
    second ApplyBoundaryOnZSGrid every substep, in the fused graph as
    ZSMPMSubstep's ZSCollider: shape ("sphere" | "plane"), dx, center,
    radius, height, extent, translation, translation_rate, scale, scale_rate,
    ypr, type.  transfer: MakeZSGrid "transfer" (apic, flip, aflip).
    cloth: optional scenes.ClothMesh run through ToZSCloth (the particles'
    model) and written back by UpdatePrimitiveFromZSParticles; the return
    value then ends with the cloth's vertex positions and velocities.
    trackers: optional (n, 3) points run through ToTrackerParticles and
    written back the same way; the return value then ends with their
    positions and velocities.  write_path: after the substeps, ComputeVonMises
    and WriteZSParticles to this .geo file.  bending: (type, stiffness) of a
    ConstructBendingSprings on the cloth, fed to the ZSBending inputs.  attr:
    (name, width) of an UpdatePrimitiveAttrFromZSParticles after the
    substeps; the attribute's values are appended to the return value.
    params: ConfigConstitutiveModel's "params" dict ({key: number}), e.g.
    {"friction_angle": 30.0} for Drucker-Prager sand.  boundary_mesh:
    optional (pos, tris, vel or None, type) of a triangle mesh made a boundary
    grid (ToBoundaryParticles, MakeZSGrid "boundary",
    ZSBoundaryPrimitiveToZSGrid) and applied after the walls and the collider
    -- by ApplyGridBoundaryOnZSGrid in the stage graph, as ZSMPMSubstep's
    BoundaryZSGrid in the fused one.  tracker_tets: optional (m, 4) tetrahedra
    over the tracker points: they then enter as a tetrahedral mesh through
    ToZSParticles (category 3) instead of ToTrackerParticles."""
    L = load_nodes()
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 3)
    v = np.ascontiguousarray(v, dtype=np.float32).reshape(-1, 3)
    n = x.shape[0]
    ox = np.zeros_like(x)
    ov = np.zeros_like(x)
    vmax = np.zeros(1, np.float32)
    err = C.create_string_buffer(1024)
    shape, lsp, lst = None, None, None
    if levelset:
        ls = levelset
        vals = ([ls.get("dx", 1.0 / 64)] + list(ls.get("center", (0.0, 0.0, 0.0))) +
                [ls.get("radius", 0.1), ls.get("height", 0.0), ls.get("extent", 0.5)] +
                list(ls.get("translation", (0.0, 0.0, 0.0))) +
                list(ls.get("translation_rate", (0.0, 0.0, 0.0))) +
                [ls.get("scale", 1.0), ls.get("scale_rate", 0.0)] + list(ls.get("ypr", (0.0, 0.0, 0.0))))
        lsp = np.asarray(vals, np.float32)
        shape = ls["shape"].encode()
        lst = ls.get("type", "sticky").encode()
    cl = {}
    if cloth is not None:
        cl["x"] = np.ascontiguousarray(cloth.x, dtype=np.float32)
        cl["v"] = None if cloth.v is None else np.ascontiguousarray(cloth.v, dtype=np.float32)
        cl["t"] = np.ascontiguousarray(cloth.tris, dtype=np.int32)
        cl["p"] = np.array([cloth.gamma, cloth.k, cloth.fa, cloth.dc], np.float32)
        cl["ox"] = np.zeros_like(cl["x"])
        cl["ov"] = np.zeros_like(cl["x"])
    aout = None
    if attr:
        aout = np.zeros((n, 3) if attr[1] == 3 else n, np.float32)
    tk = {}
    if trackers is not None:
        tk["x"] = np.ascontiguousarray(trackers, dtype=np.float32).reshape(-1, 3)
        tk["ox"] = np.zeros_like(tk["x"])
        tk["ov"] = np.zeros_like(tk["x"])
    tq = None if tracker_tets is None else np.ascontiguousarray(tracker_tets, np.int32).reshape(-1, 4)
    bm = {}
    if boundary_mesh is not None:
        bm["x"] = np.ascontiguousarray(boundary_mesh[0], dtype=np.float32).reshape(-1, 3)
        bm["t"] = np.ascontiguousarray(boundary_mesh[1], dtype=np.int32).reshape(-1, 3)
        bm["v"] = (None if boundary_mesh[2] is None else
                   np.ascontiguousarray(boundary_mesh[2], dtype=np.float32).reshape(-1, 3))
        bm["type"] = boundary_mesh[3].encode()
    rc = L.zsn_run_graph(1 if fused else 0, n, _p(x), _p(v), dx, type.encode(),
                         plasticity.encode(), E, nu, density, ppc, bc.encode(), thickness, dt,
                         gravity, substeps, _p(ox), _p(ov), _p(vmax), err, 1024, shape,
                         _p(lsp) if lsp is not None else None, lst, transfer.encode(),
                         cl["x"].shape[0] if cl else 0, _p(cl.get("x")), _p(cl.get("v")),
                         cl["t"].shape[0] if cl else 0, _p(cl.get("t")), _p(cl.get("p")),
                         _p(cl.get("ox")), _p(cl.get("ov")),
                         tk["x"].shape[0] if tk else 0, _p(tk.get("x")), _p(tk.get("ox")),
                         _p(tk.get("ov")), write_path.encode() if write_path else None,
                         bending[0].encode() if bending else None,
                         float(bending[1]) if bending else 0.0,
                         attr[0].encode() if attr else None, int(attr[1]) if attr else 0,
                         _p(aout),
                         ";".join(f"{k}={float(v)!r}" for k, v in (params or {}).items()).encode(),
                         bm["x"].shape[0] if bm else 0, _p(bm.get("x")), _p(bm.get("v")),
                         bm["t"].shape[0] if bm else 0, _p(bm.get("t")), bm.get("type"),
                         tq.shape[0] if tq is not None else 0, _p(tq))
    if rc != 0:
        raise RuntimeError(err.value.decode())
    out = (ox, ov, float(vmax[0]))
    if cl:
        out += (cl["ox"], cl["ov"])
    if tk:
        out += (tk["ox"], tk["ov"])
    if attr:
        out += (aout,)
    return out
