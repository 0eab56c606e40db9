"""ctypes binding of the C ABI in include/gtc.h (libgtc.so, built in-tree).

The Python face of the CUDA backend: the same calls a C++ caller makes
through gtc.hpp, with numpy arrays on the host and raw device pointers for
the ``*_device`` forms. Errors raise ``GtcInvalidArgument`` (a ValueError,
the reference's std::invalid_argument) or ``GtcError`` (a RuntimeError, the
reference's std::runtime_error). There is no CPU fallback: if libgtc.so is
missing, importing this module fails.
"""

import ctypes as C
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libgtc.so"

GTC_OK, GTC_INVALID_ARGUMENT, GTC_RUNTIME_ERROR, GTC_NO_DEVICE, GTC_OUT_OF_MEMORY = range(5)
CRITERION_THETA, CRITERION_LEARNED = 0, 1


class GtcError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class GtcInvalidArgument(GtcError, ValueError):
    pass


class GravityParams(C.Structure):
    _fields_ = [("G", C.c_double), ("theta", C.c_double), ("eps", C.c_double),
                ("quadrupole", C.c_int32), ("group_size", C.c_int32), ("leaf_size", C.c_int32),
                ("pack", C.c_int32), ("criterion", C.c_int32), ("reserved", C.c_int32),
                ("alpha", C.c_double)]


class Diagnostics(C.Structure):
    _fields_ = [("time", C.c_double), ("kinetic", C.c_double), ("potential", C.c_double),
                ("total", C.c_double), ("virial_ratio", C.c_double),
                ("momentum", C.c_double * 3), ("angular_momentum", C.c_double * 3),
                ("centre_of_mass", C.c_double * 3)]


SOLVER_GROUP, SOLVER_DIRECT = 0, 1


class KernelParams(C.Structure):
    _fields_ = [("n", C.c_uint32), ("n_groups", C.c_uint32), ("G", C.c_float),
                ("eps2", C.c_float), ("quadrupole", C.c_uint32), ("pad", C.c_uint32 * 3)]


class Stats(C.Structure):
    _fields_ = [("tree_ms", C.c_double), ("lists_ms", C.c_double), ("evaluate_ms", C.c_double),
                ("total_ms", C.c_double), ("cell_interactions", C.c_uint64),
                ("body_interactions", C.c_uint64), ("max_list", C.c_uint64),
                ("n_cell_list", C.c_uint64), ("n_body_list", C.c_uint64),
                ("n_nodes", C.c_uint32), ("n_groups", C.c_uint32), ("max_group", C.c_uint32),
                ("depth", C.c_uint32), ("eval_kernel_ms", C.c_double),
                ("kernel_launches", C.c_uint64), ("walk_tests_fp64", C.c_uint64),
                ("mlp_rows", C.c_uint64), ("mlp_batches", C.c_uint64),
                ("criterion_used", C.c_uint32), ("graph_steps", C.c_uint32),
                ("list_passes", C.c_uint32), ("spilled_groups", C.c_uint32),
                ("walk_nodes", C.c_uint64)]


class StageTimes(C.Structure):
    _fields_ = [("build_ms", C.c_double), ("keys_ms", C.c_double), ("sort_ms", C.c_double),
                ("topology_ms", C.c_double), ("moments_ms", C.c_double),
                ("walk_ms", C.c_double), ("sort_passes", C.c_uint32), ("reserved", C.c_uint32),
                ("quad_ms", C.c_double)]


NODE_DTYPE = np.dtype([
    ("center", "<f8", 3), ("half", "<f8"), ("com", "<f8", 3), ("mass", "<f8"),
    ("quad", "<f8", 6), ("delta", "<f8"), ("begin", "<u4"), ("end", "<u4"), ("skip", "<u4"),
    ("parent", "<u4"), ("depth", "<i4"), ("n_children", "<i4")])
assert NODE_DTYPE.itemsize == 144

assert C.sizeof(GravityParams) == 56 and C.sizeof(KernelParams) == 32 and C.sizeof(Stats) == 152

# Learned criterion model: W1[6][64], b1[64], W2[64][64], b2[64], W3[64], b3,
# then feature mean[6], std[6], y_mean, y_std, band (include/gtc.h).
LEARNED_FEATURES, LEARNED_PARAMS, LEARNED_MODEL_FLOATS = 6, 4673, 4688


def _load():
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is not built: run __graft_entry__.build() (make -C "
                          "galactic-tides_gb300)")
    lib = C.CDLL(str(LIB_PATH))
    V, I, U32, U64, D = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_double
    P = C.c_void_p
    sig = {
        "gtc_create": (I, [C.POINTER(V), I]),
        "gtc_destroy": (None, [V]),
        "gtc_last_error": (C.c_char_p, [V]),
        "gtc_status_name": (C.c_char_p, [I]),
        "gtc_stream": (V, [V]),
        "gtc_direct": (I, [V, P, C.POINTER(KernelParams), P]),
        "gtc_tree": (I, [V, P, P, U32, P, U64, P, U64, P, C.POINTER(KernelParams), P]),
        "gtc_group_force": (I, [V, P, P, U64, C.POINTER(GravityParams), P, P]),
        "gtc_group_force_device": (I, [V, P, P, U64, C.POINTER(GravityParams), P, P]),
        "gtc_direct_force": (I, [V, P, P, U64, C.POINTER(GravityParams), P, P]),
        "gtc_direct_force_device": (I, [V, P, P, U64, C.POINTER(GravityParams), P, P]),
        "gtc_direct_fp64_device": (I, [V, P, P, U64, P, U64, D, D, P, P]),
        "gtc_tree_force": (I, [V, P, P, U64, C.POINTER(GravityParams), P, P]),
        "gtc_tree_force_device": (I, [V, P, P, U64, C.POINTER(GravityParams), P, P]),
        "gtc_get_stats": (I, [V, C.POINTER(Stats)]),
        "gtc_sample_indices": (None, [U64, U64, U64, P]),
        "gtc_get_stage_times": (I, [V, C.POINTER(StageTimes)]),
        "gtc_write_snapshot": (I, [C.c_char_p, U64, P, P, P, P, P, P, D, C.c_char_p]),
        "gtc_snapshot_info": (I, [C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_double), P,
                                  C.POINTER(C.c_uint64)]),
        "gtc_read_snapshot": (I, [C.c_char_p, U64, P, P, P, P, P, P, P]),
        "gtc_measure_fp32_peak": (I, [V, C.POINTER(C.c_double)]),
        "gtc_set_option": (I, [V, C.c_char_p, D]),
        "gtc_learned_add_samples": (I, [V, P, P, U64, C.POINTER(GravityParams), D, D, U64, U32,
                                        C.POINTER(C.c_uint64)]),
        "gtc_learned_sample_count": (I, [V, C.POINTER(C.c_uint64)]),
        "gtc_learned_export_samples": (I, [V, U64, U64, P, P, P]),
        "gtc_learned_clear_samples": (I, [V]),
        "gtc_learned_train": (I, [V, U64, U32, C.c_float, U64, I, C.POINTER(C.c_double)]),
        "gtc_learned_gradient": (I, [V, P, P, P, U32, P, C.POINTER(C.c_double)]),
        "gtc_learned_set_model": (I, [V, P]),
        "gtc_learned_get_model": (I, [V, P]),
        "gtc_learned_predict": (I, [V, P, U64, P]),
        "gtc_direct_fp64_noalloc": (I, [P, P, U64, P, U64, D, D, P, P, V]),
        "gtc_leapfrog_device": (I, [V, P, P, P, P, P, U64, C.POINTER(GravityParams), I, D, U64,
                                    I, I]),
        "gtc_diagnostics_device": (I, [V, P, P, P, P, U64, D, C.POINTER(Diagnostics)]),
        "gtc_ensemble_create": (I, [C.POINTER(V), I, U32]),
        "gtc_ensemble_destroy": (None, [V]),
        "gtc_ensemble_last_error": (C.c_char_p, [V]),
        "gtc_ensemble_set_system": (I, [V, U32, P, P, P, P, P, U64, C.POINTER(GravityParams)]),
        "gtc_ensemble_leapfrog": (I, [V, D, U64, I, I]),
        "gtc_ensemble_context": (V, [V, U32]),
        "gtc_ensemble_set_option": (I, [V, C.c_char_p, D]),
        "gtc_autotune_group": (I, [V, P, P, U64, C.POINTER(GravityParams),
                                   C.POINTER(GravityParams), C.POINTER(C.c_double),
                                   C.POINTER(C.c_int)]),
        "gtc_autotune_direct": (I, [V, P, P, U64, C.POINTER(GravityParams), C.POINTER(C.c_int),
                                    C.POINTER(C.c_double)]),
        "gtc_autotune_eval": (I, [V, P, P, U64, C.POINTER(GravityParams), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.POINTER(C.c_double)]),
        "gtc_group_sizes": (I, [V] + [C.POINTER(C.c_uint64)] * 5),
        "gtc_group_export": (I, [V, P, P, P, P, P, P, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def gravity_params(G=1.0, theta=0.75, eps=0.025, quadrupole=True, group_size=32, leaf_size=8,
                   pack=True, criterion=CRITERION_THETA, alpha=0.0):
    return GravityParams(G, theta, eps, int(quadrupole), group_size, leaf_size, int(pack),
                         criterion, 0, alpha)


def direct_fp64_noalloc(pos_ptr, mass_ptr, n, idx_ptr, m, acc_ptr, pot_ptr, G=1.0, eps=0.025,
                        stream=None):
    """gtc_direct_fp64_noalloc: FP64 sampled sums with no allocation and no
    context, enqueued on `stream` (a cudaStream_t handle, None for the default
    stream); the caller synchronizes."""
    rc = lib.gtc_direct_fp64_noalloc(pos_ptr, mass_ptr, n, idx_ptr, m, G, eps, acc_ptr, pot_ptr,
                                     stream)
    if rc != GTC_OK:
        raise (GtcInvalidArgument if rc == GTC_INVALID_ARGUMENT else GtcError)(
            rc, lib.gtc_last_error(None).decode())


class Context:
    """One gtc_context: a device, a CUDA stream, and buffers reused between calls."""

    def __init__(self, device=0):
        h = C.c_void_p()
        rc = lib.gtc_create(C.byref(h), device)
        if rc != GTC_OK:
            raise (GtcInvalidArgument if rc == GTC_INVALID_ARGUMENT else GtcError)(
                rc, lib.gtc_last_error(None).decode())
        self.h = h

    def close(self):
        if self.h:
            lib.gtc_destroy(self.h)
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

    def _check(self, rc):
        if rc != GTC_OK:
            msg = lib.gtc_last_error(self.h).decode()
            raise (GtcInvalidArgument if rc == GTC_INVALID_ARGUMENT else GtcError)(rc, msg)

    @property
    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        return lib.gtc_stream(self.h)

    # ---- reference-facing calls with host arrays -----------------------------

    def group_force(self, pos, mass, **kw):
        """GroupTreeGravity(Device::CUDA).compute: host arrays in, (acc, pot) out."""
        pos = _f64(pos, (-1, 3))
        mass = _f64(mass)
        n = mass.shape[0]
        acc = np.empty((n, 3))
        pot = np.empty(n)
        gp = gravity_params(**kw)
        self._check(lib.gtc_group_force(self.h, _ptr(pos), _ptr(mass), n, C.byref(gp),
                                        _ptr(acc), _ptr(pot)))
        return acc, pot

    def direct_force(self, pos, mass, **kw):
        """DirectGravity(Device::CUDA).compute: FP32 direct sum, host arrays."""
        pos = _f64(pos, (-1, 3))
        mass = _f64(mass)
        n = mass.shape[0]
        acc = np.empty((n, 3))
        pot = np.empty(n)
        gp = gravity_params(**kw)
        self._check(lib.gtc_direct_force(self.h, _ptr(pos), _ptr(mass), n, C.byref(gp),
                                         _ptr(acc), _ptr(pot)))
        return acc, pot

    def tree_force(self, pos, mass, **kw):
        """compute_gravity_tree on the device (Octree::accel_pot per body,
        FP64), host arrays."""
        pos = _f64(pos, (-1, 3))
        mass = _f64(mass)
        n = mass.shape[0]
        acc = np.empty((n, 3))
        pot = np.empty(n)
        gp = gravity_params(**kw)
        self._check(lib.gtc_tree_force(self.h, _ptr(pos), _ptr(mass), n, C.byref(gp), _ptr(acc),
                                       _ptr(pot)))
        return acc, pot

    def direct(self, bodies, G=1.0, eps2=0.0):
        """metal::Context::direct: float4 bodies -> float4 (ax, ay, az, pot)."""
        bodies = np.ascontiguousarray(bodies, dtype=np.float32).reshape(-1, 4)
        n = bodies.shape[0]
        out = np.empty((n, 4), np.float32)
        kp = KernelParams(n, 0, G, eps2, 0, (C.c_uint32 * 3)())
        self._check(lib.gtc_direct(self.h, _ptr(bodies), C.byref(kp), _ptr(out)))
        return out

    def tree(self, bodies, cells, cell_list, body_list, groups, G=1.0, eps2=0.0,
             quadrupole=True, n_groups=None):
        """metal::Context::tree: evaluate given grouped lists -> float4 per body (tree order)."""
        bodies = np.ascontiguousarray(bodies, dtype=np.float32).reshape(-1, 4)
        cells = np.ascontiguousarray(cells, dtype=np.float32).reshape(-1, 12)
        cl = np.ascontiguousarray(cell_list, dtype=np.uint32)
        bl = np.ascontiguousarray(body_list, dtype=np.uint32)
        groups = np.ascontiguousarray(groups, dtype=np.uint32).reshape(-1, 8)
        n = bodies.shape[0]
        ng = groups.shape[0] if n_groups is None else n_groups
        out = np.empty((n, 4), np.float32)
        kp = KernelParams(n, ng, G, eps2, int(quadrupole), (C.c_uint32 * 3)())
        self._check(lib.gtc_tree(self.h, _ptr(bodies), _ptr(cells), cells.shape[0], _ptr(cl),
                                 cl.shape[0], _ptr(bl), bl.shape[0], _ptr(groups), C.byref(kp),
                                 _ptr(out)))
        return out

    # ---- device-pointer forms ------------------------------------------------

    def group_force_device(self, pos_ptr, mass_ptr, n, acc_ptr, pot_ptr, **kw):
        gp = gravity_params(**kw)
        self._check(lib.gtc_group_force_device(self.h, pos_ptr, mass_ptr, n, C.byref(gp),
                                               acc_ptr, pot_ptr))

    def direct_force_device(self, pos_ptr, mass_ptr, n, acc_ptr, pot_ptr, **kw):
        gp = gravity_params(**kw)
        self._check(lib.gtc_direct_force_device(self.h, pos_ptr, mass_ptr, n, C.byref(gp),
                                                acc_ptr, pot_ptr))

    def direct_fp64_device(self, pos_ptr, mass_ptr, n, idx_ptr, m, acc_ptr, pot_ptr, G=1.0,
                           eps=0.025):
        self._check(lib.gtc_direct_fp64_device(self.h, pos_ptr, mass_ptr, n, idx_ptr, m, G, eps,
                                               acc_ptr, pot_ptr))

    # ---- introspection -----------------------------------------------------

    def set_option(self, name, value):
        self._check(lib.gtc_set_option(self.h, name.encode(), float(value)))

    # ---- tuning ----------------------------------------------------------------

    def autotune_group(self, pos_ptr, mass_ptr, n, **kw):
        """gtc_autotune_group -> (group_size, pack (0 off, 1 a group's worth,
        k >= 2 the packing threshold), ms per evaluation, walk_warps)."""
        base = gravity_params(**kw)
        best = GravityParams()
        ms = C.c_double()
        walk = C.c_int()
        self._check(lib.gtc_autotune_group(self.h, pos_ptr, mass_ptr, n, C.byref(base),
                                           C.byref(best), C.byref(ms), C.byref(walk)))
        return best.group_size, best.pack, ms.value, walk.value

    def autotune_direct(self, pos_ptr, mass_ptr, n, **kw):
        """gtc_autotune_direct -> (targets per thread, kernel ms); the context
        keeps the winner."""
        gp = gravity_params(**kw)
        k, ms = C.c_int(), C.c_double()
        self._check(lib.gtc_autotune_direct(self.h, pos_ptr, mass_ptr, n, C.byref(gp),
                                            C.byref(k), C.byref(ms)))
        return k.value, ms.value

    def autotune_eval(self, pos_ptr, mass_ptr, n, **kw):
        """gtc_autotune_eval -> (staged pairs per iteration, pass cost,
        evaluation kernel ms); the context keeps the winner."""
        gp = gravity_params(**kw)
        k, c, ms = C.c_int(), C.c_int(), C.c_double()
        self._check(lib.gtc_autotune_eval(self.h, pos_ptr, mass_ptr, n, C.byref(gp),
                                          C.byref(k), C.byref(c), C.byref(ms)))
        return k.value, c.value, ms.value

    # ---- time integration ------------------------------------------------------

    def leapfrog_device(self, pos_ptr, vel_ptr, mass_ptr, acc_ptr, pot_ptr, n, dt, steps,
                        prime=True, graph=False, solver=SOLVER_GROUP, **kw):
        """LeapfrogKDK on device arrays: optional prime(), then `steps` KDK steps."""
        gp = gravity_params(**kw)
        self._check(lib.gtc_leapfrog_device(self.h, pos_ptr, vel_ptr, mass_ptr, acc_ptr,
                                            pot_ptr, n, C.byref(gp), solver, dt, steps,
                                            int(prime), int(graph)))

    def diagnostics_device(self, pos_ptr, vel_ptr, mass_ptr, pot_ptr, n, time=0.0):
        d = Diagnostics()
        self._check(lib.gtc_diagnostics_device(self.h, pos_ptr, vel_ptr, mass_ptr, pot_ptr, n,
                                               time, C.byref(d)))
        out = {k: getattr(d, k) for k, _ in Diagnostics._fields_}
        for k in ("momentum", "angular_momentum", "centre_of_mass"):
            out[k] = list(out[k])
        return out

    # ---- learned opening criterion -------------------------------------------

    def learned_add_samples(self, pos, mass, theta_gen=0.5, theta_guard=1.5, max_new=1 << 20,
                            max_cell_bodies=8192, **kw):
        """Labelled (group, cell) samples from these bodies -> number added."""
        pos = _f64(pos, (-1, 3))
        mass = _f64(mass)
        gp = gravity_params(**kw)
        added = C.c_uint64()
        self._check(lib.gtc_learned_add_samples(self.h, _ptr(pos), _ptr(mass), mass.shape[0],
                                                C.byref(gp), theta_gen, theta_guard, max_new,
                                                max_cell_bodies, C.byref(added)))
        return added.value

    def learned_sample_count(self):
        v = C.c_uint64()
        self._check(lib.gtc_learned_sample_count(self.h, C.byref(v)))
        return v.value

    def learned_samples(self, first=0, count=None):
        """-> (features (count, 6), labels (count,), (group, node) pairs (count, 2))."""
        if count is None:
            count = self.learned_sample_count() - first
        feat = np.empty((count, LEARNED_FEATURES), np.float32)
        label = np.empty(count, np.float32)
        pairs = np.empty((count, 2), np.uint32)
        self._check(lib.gtc_learned_export_samples(self.h, first, count, _ptr(feat),
                                                   _ptr(label), _ptr(pairs)))
        return feat, label, pairs

    def learned_clear_samples(self):
        self._check(lib.gtc_learned_clear_samples(self.h))

    def learned_train(self, steps, batch=4096, lr=1e-3, seed=1, init=False):
        loss = C.c_double()
        self._check(lib.gtc_learned_train(self.h, steps, batch, lr, seed, int(init),
                                          C.byref(loss)))
        return loss.value

    def learned_gradient(self, model, feat, label):
        """Gradient (LEARNED_PARAMS,) and loss of `model` on the given samples."""
        model = np.ascontiguousarray(model, np.float32)
        feat = np.ascontiguousarray(feat, np.float32).reshape(-1, LEARNED_FEATURES)
        label = np.ascontiguousarray(label, np.float32)
        grad = np.empty(LEARNED_PARAMS, np.float32)
        loss = C.c_double()
        self._check(lib.gtc_learned_gradient(self.h, _ptr(model), _ptr(feat), _ptr(label),
                                             label.shape[0], _ptr(grad), C.byref(loss)))
        return grad, loss.value

    def learned_set_model(self, model):
        model = np.ascontiguousarray(model, np.float32)
        if model.shape != (LEARNED_MODEL_FLOATS,):
            raise ValueError(f"a model has {LEARNED_MODEL_FLOATS} floats")
        self._check(lib.gtc_learned_set_model(self.h, _ptr(model)))

    def learned_get_model(self):
        model = np.empty(LEARNED_MODEL_FLOATS, np.float32)
        self._check(lib.gtc_learned_get_model(self.h, _ptr(model)))
        return model

    def learned_predict(self, feat):
        feat = np.ascontiguousarray(feat, np.float32).reshape(-1, LEARNED_FEATURES)
        pred = np.empty(feat.shape[0], np.float32)
        self._check(lib.gtc_learned_predict(self.h, _ptr(feat), feat.shape[0], _ptr(pred)))
        return pred

    def fp32_peak_tflops(self):
        v = C.c_double()
        self._check(lib.gtc_measure_fp32_peak(self.h, C.byref(v)))
        return v.value

    def stage_times(self):
        """Per-stage device times of the last eager group solve (option
        stage_events = 1), ms; -1 where a stage was not timed."""
        st = StageTimes()
        self._check(lib.gtc_get_stage_times(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in StageTimes._fields_ if k != "reserved"}

    def stats(self):
        st = Stats()
        self._check(lib.gtc_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in Stats._fields_}

    def export(self):
        """Tree, groups and lists of the last group_force, as numpy arrays."""
        sz = [C.c_uint64() for _ in range(5)]
        self._check(lib.gtc_group_sizes(self.h, *[C.byref(x) for x in sz]))
        n, m, ng, ncl, nbl = (x.value for x in sz)
        nodes = np.zeros(m, NODE_DTYPE)
        order = np.zeros(n, np.uint64)
        bodies = np.zeros((n, 4), np.float32)
        cells = np.zeros((m, 12), np.float32)
        groups = np.zeros((ng, 8), np.uint32)
        cl = np.zeros(ncl, np.uint32)
        bl = np.zeros(nbl, np.uint32)
        out = np.zeros((n, 4), np.float32)
        self._check(lib.gtc_group_export(self.h, _ptr(nodes), _ptr(order), _ptr(bodies),
                                         _ptr(cells), _ptr(groups), _ptr(cl), _ptr(bl),
                                         _ptr(out)))
        return dict(nodes=nodes, order=order, bodies=bodies, cells=cells, groups=groups,
                    cell_list=cl, body_list=bl, out=out)


# ---- inputs ------------------------------------------------------------------

# the synthetic galaxies live in galaxy.py (pure numpy); re-exported here
from .galaxy import (GalaxyModel, galaxy_model, make_encounter, make_galaxy,  # noqa: E402,F401
                     orient, parabolic_orbit)


# ---- snapshots (raw binary; the reference's GADGET HDF5 content) -------------

def _check_free(rc):
    if rc != GTC_OK:
        msg = lib.gtc_last_error(None).decode()
        raise (GtcInvalidArgument if rc == GTC_INVALID_ARGUMENT else GtcError)(rc, msg)


def write_snapshot(path, pos, vel, mass, ids=None, types=None, pot=None, time=0.0,
                   metadata=None):
    """Writes a snapshot (gtc_write_snapshot); metadata: a dict of strings."""
    pos = np.ascontiguousarray(pos, np.float64)
    vel = np.ascontiguousarray(vel, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    n = mass.shape[0]
    ids = None if ids is None else np.ascontiguousarray(ids, np.uint64)
    types = None if types is None else np.ascontiguousarray(types, np.uint8)
    pot = None if pot is None else np.ascontiguousarray(pot, np.float64)
    meta = "".join(f"{k}={v}\n" for k, v in (metadata or {}).items()).encode()
    p = lambda a: None if a is None else _ptr(a)
    _check_free(lib.gtc_write_snapshot(str(path).encode(), n, _ptr(pos), _ptr(vel), _ptr(mass),
                                       p(ids), p(types), p(pot), float(time), meta))


def read_snapshot(path):
    """-> dict(pos, vel, mass, ids, types, pot, time, count_by_type, metadata)."""
    n, t, mb = C.c_uint64(), C.c_double(), C.c_uint64()
    counts = np.zeros(6, np.uint64)
    path = str(path).encode()
    _check_free(lib.gtc_snapshot_info(path, C.byref(n), C.byref(t), _ptr(counts), C.byref(mb)))
    n = n.value
    out = dict(pos=np.empty((n, 3)), vel=np.empty((n, 3)), mass=np.empty(n),
               ids=np.empty(n, np.uint64), types=np.empty(n, np.uint8), pot=np.empty(n))
    meta = C.create_string_buffer(max(1, mb.value))
    _check_free(lib.gtc_read_snapshot(path, n, _ptr(out["pos"]), _ptr(out["vel"]),
                                      _ptr(out["mass"]), _ptr(out["ids"]), _ptr(out["types"]),
                                      _ptr(out["pot"]), meta))
    text = meta.raw[:mb.value].decode()
    out.update(time=t.value, count_by_type=counts,
               metadata=dict(line.split("=", 1) for line in text.splitlines() if "=" in line))
    return out


def sample_indices(n, m=4096, seed=1):
    """The reference bench's accuracy sample: mt19937_64(seed) shuffle, first m."""
    out = np.empty(min(n, m), np.uint64)
    lib.gtc_sample_indices(n, m, seed, _ptr(out))
    return out


class _Borrowed(Context):
    """A context owned by an ensemble (not destroyed by this object)."""

    def __init__(self, handle):
        self.h = handle

    def close(self):
        self.h = None


class Ensemble:
    """gtc_ensemble: independent systems advanced together (device arrays)."""

    def __init__(self, systems, device=0):
        h = C.c_void_p()
        rc = lib.gtc_ensemble_create(C.byref(h), device, systems)
        if rc != GTC_OK:
            raise (GtcInvalidArgument if rc == GTC_INVALID_ARGUMENT else GtcError)(
                rc, lib.gtc_ensemble_last_error(None).decode())
        self.h = h
        self.systems = systems

    def _check(self, rc):
        if rc != GTC_OK:
            msg = lib.gtc_ensemble_last_error(self.h).decode()
            raise (GtcInvalidArgument if rc == GTC_INVALID_ARGUMENT else GtcError)(rc, msg)

    def set_system(self, i, pos_ptr, vel_ptr, mass_ptr, acc_ptr, pot_ptr, n, **kw):
        gp = gravity_params(**kw)
        self._check(lib.gtc_ensemble_set_system(self.h, i, pos_ptr, vel_ptr, mass_ptr, acc_ptr,
                                                pot_ptr, n, C.byref(gp)))

    def leapfrog(self, dt, steps, prime=True, graph=True):
        self._check(lib.gtc_ensemble_leapfrog(self.h, dt, steps, int(prime), int(graph)))

    def context(self, i):
        return _Borrowed(lib.gtc_ensemble_context(self.h, i))

    def set_option(self, name, value):
        """Ensemble options: "forest" (-1 when eligible, 0 never, 1 always)
        and "walk_warps" (the forest walk: -1 by group count, 0, 1)."""
        self._check(lib.gtc_ensemble_set_option(self.h, name.encode(), float(value)))

    def close(self):
        if self.h:
            lib.gtc_ensemble_destroy(self.h)
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
