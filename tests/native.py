"""ctypes bindings for the test-side native libraries.

* ``Oracle``  -- oracle/liboracle.so, the CPU restatement of the reference's
  hot path (the checker).
* ``Ref``     -- oracle/_ref/libgtref.so, the reference's own sources built by
  oracle/Makefile.ref; only present where the reference tree is on disk.

Node arrays come back as numpy structured arrays with the field order of
``Octree::Node`` (include/galactic_tides/octree.h:52-63).
"""

import ctypes as C
import os
import pathlib

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
ORACLE_SO = ROOT / "oracle" / "liboracle.so"
REF_SO = ROOT / "oracle" / "_ref" / "libgtref.so"

NODE_DTYPE = np.dtype([
    ("center", "<f8", 3), ("half", "<f8"), ("com", "<f8", 3), ("mass", "<f8"),
    ("quad", "<f8", 6), ("delta", "<f8"), ("first_child", "<i4"), ("n_children", "<i4"),
    ("begin", "<u4"), ("end", "<u4")])
assert NODE_DTYPE.itemsize == 136

NO_PARALLEL = (1 << 62)   # parallel_threshold that keeps the serial layout


def _p(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class ListStats(C.Structure):
    _fields_ = [("n_groups", C.c_uint64), ("n_cell_list", C.c_uint64), ("n_body_list", C.c_uint64),
                ("cell_interactions", C.c_uint64), ("body_interactions", C.c_uint64),
                ("max_list", C.c_uint64), ("max_group", C.c_int64), ("origin", C.c_double * 3)]


class Lists:
    """Flat grouped interaction lists, in the layout of GroupLists (group_lists.h:37-55)."""

    def __init__(self, stats, bodies, cells, cell_list, body_list, groups):
        self.stats = stats
        self.bodies = bodies          # (n, 4) float32, tree order
        self.cells = cells            # (n_nodes, 12) float32
        self.cell_list = cell_list    # uint32
        self.body_list = body_list    # uint32
        self.groups = groups          # (n_groups, 8) uint32

    @property
    def n_groups(self):
        return self.groups.shape[0]


class _Common:
    """Entry points the oracle and the reference shim share."""

    def __init__(self, lib, prefix):
        self.lib = lib
        self.prefix = prefix
        L = lib
        V, D, U64, I = C.c_void_p, C.c_double, C.c_uint64, C.c_int
        pD, pF, pU32, pU64 = (C.POINTER(C.c_double), C.POINTER(C.c_float),
                              C.POINTER(C.c_uint32), C.POINTER(C.c_uint64))
        self._f = {}
        def fn(name, res, args):
            f = getattr(L, prefix + name)
            f.restype = res
            f.argtypes = args
            self._f[name] = f
        fn("last_error", C.c_char_p, [])
        fn("tree_build", V, [pD, pD, U64, I, U64])
        fn("tree_free", None, [V])
        fn("tree_nnodes", U64, [V])
        fn("tree_depth", I, [V])
        fn("tree_export", None, [V, C.c_void_p, pU64])
        fn("lists_free", None, [V])
        fn("lists_stats", None, [V, C.POINTER(ListStats)])
        fn("lists_export", None, [V, pF, pF, pU32, pU32, pU32])

    def error(self):
        return self._f["last_error"]().decode()

    def tree(self, pos, mass, leaf_size=8, parallel_threshold=NO_PARALLEL):
        """Octree::build -> (nodes structured array, order uint64, depth)."""
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        h = self._f["tree_build"](_p(pos, C.c_double), _p(mass, C.c_double), n, leaf_size,
                                  parallel_threshold)
        if not h:
            raise RuntimeError(self.error())
        try:
            nn = self._f["tree_nnodes"](h)
            nodes = np.zeros(nn, dtype=NODE_DTYPE)
            order = np.zeros(n, dtype=np.uint64)
            self._f["tree_export"](h, nodes.ctypes.data, _p(order, C.c_uint64))
            return nodes, order, self._f["tree_depth"](h)
        finally:
            self._f["tree_free"](h)

    def _export_lists(self, lh, n, n_nodes):
        st = ListStats()
        self._f["lists_stats"](lh, C.byref(st))
        bodies = np.zeros((n, 4), np.float32)
        cells = np.zeros((n_nodes, 12), np.float32)
        cl = np.zeros(st.n_cell_list, np.uint32)
        bl = np.zeros(st.n_body_list, np.uint32)
        groups = np.zeros((st.n_groups, 8), np.uint32)
        self._f["lists_export"](lh, _p(bodies, C.c_float), _p(cells, C.c_float),
                                _p(cl, C.c_uint32), _p(bl, C.c_uint32), _p(groups, C.c_uint32))
        return Lists(st, bodies, cells, cl, bl, groups)


class Oracle(_Common):
    def __init__(self, path=ORACLE_SO):
        super().__init__(C.CDLL(str(path)), "orc_")
        L = self.lib
        V, D, U64, I = C.c_void_p, C.c_double, C.c_uint64, C.c_int
        pD, pF, pU32, pU64 = (C.POINTER(C.c_double), C.POINTER(C.c_float),
                              C.POINTER(C.c_uint32), C.POINTER(C.c_uint64))
        L.orc_lists_build.restype = V
        L.orc_lists_build.argtypes = [V, D, I, I]
        L.orc_eval_lists.restype = None
        L.orc_eval_lists.argtypes = [pF, U64, pF, pU32, pU32, pU32, U64, D, D, I, pF]
        L.orc_group_force.restype = I
        L.orc_group_force.argtypes = [pD, pD, U64, D, D, D, I, I, I, I, I, U64, pD, pD, V]
        L.orc_tree_force.restype = I
        L.orc_tree_force.argtypes = [pD, pD, U64, D, D, D, I, I, U64, pD, pD, pU64]
        L.orc_direct_fp64.restype = None
        L.orc_direct_fp64.argtypes = [pD, pD, U64, pU64, U64, D, D, pD, pD]
        L.orc_pack_bodies.restype = None
        L.orc_pack_bodies.argtypes = [pD, pD, U64, pD, pF]
        L.orc_direct_fp32.restype = None
        L.orc_direct_fp32.argtypes = [pF, U64, pU64, U64, D, D, pF]
        L.orc_tree_accel_pot.restype = None
        L.orc_tree_accel_pot.argtypes = [V, pD, U64, D, D, D, I, pD, pD]
        L.orc_leapfrog_group.restype = I
        L.orc_leapfrog_group.argtypes = [pD, pD, pD, U64, D, D, D, I, I, I, D, I, pD]
        L.orc_threads.restype = I

    def threads(self):
        return self.lib.orc_threads()

    def lists(self, pos, mass, theta=0.75, group_size=32, leaf_size=8, pack=True,
              parallel_threshold=NO_PARALLEL):
        """Octree::build + build_group_lists -> (nodes, order, Lists)."""
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        L = self.lib
        th = L.orc_tree_build(_p(pos, C.c_double), _p(mass, C.c_double), n, leaf_size,
                              parallel_threshold)
        if not th:
            raise RuntimeError(self.error())
        try:
            nn = L.orc_tree_nnodes(th)
            nodes = np.zeros(nn, dtype=NODE_DTYPE)
            order = np.zeros(n, dtype=np.uint64)
            L.orc_tree_export(th, nodes.ctypes.data, _p(order, C.c_uint64))
            lh = L.orc_lists_build(th, theta, group_size, int(pack))
            if not lh:
                raise RuntimeError(self.error())
            try:
                return nodes, order, self._export_lists(lh, n, nn)
            finally:
                L.orc_lists_free(lh)
        finally:
            L.orc_tree_free(th)

    def eval_lists(self, lists, G=1.0, eps=0.025, quadrupole=True):
        n = lists.bodies.shape[0]
        out = np.zeros((n, 4), np.float32)
        self.lib.orc_eval_lists(_p(lists.bodies, C.c_float), n, _p(lists.cells, C.c_float),
                                _p(lists.cell_list, C.c_uint32), _p(lists.body_list, C.c_uint32),
                                _p(np.ascontiguousarray(lists.groups), C.c_uint32),
                                lists.n_groups, G, eps, int(quadrupole), _p(out, C.c_float))
        return out

    def group_force(self, pos, mass, G=1.0, theta=0.75, eps=0.025, quadrupole=True,
                    group_size=32, leaf_size=8, pack=False, repeat=1,
                    parallel_threshold=20000):
        """GroupTreeGravity(Device::CPU).compute -> (acc (n,3), pot (n,), timings dict)."""
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        acc = np.zeros((n, 3))
        pot = np.zeros(n)
        tm = (C.c_double * 4 + C.c_uint64 * 2)() if False else None
        buf = np.zeros(6, dtype=np.float64)
        rc = self.lib.orc_group_force(_p(pos, C.c_double), _p(mass, C.c_double), n, G, theta,
                                      eps, int(quadrupole), group_size, leaf_size, int(pack),
                                      repeat, parallel_threshold, _p(acc, C.c_double),
                                      _p(pot, C.c_double), buf.ctypes.data)
        if rc:
            raise RuntimeError(self.error())
        ints = buf[4:].view(np.uint64)
        t = dict(tree=buf[0], lists=buf[1], evaluate=buf[2], total=buf[3],
                 cell_interactions=int(ints[0]), body_interactions=int(ints[1]))
        return acc, pot, t

    def tree_force(self, pos, mass, G=1.0, theta=0.75, eps=0.025, quadrupole=True, leaf_size=8,
                   parallel_threshold=20000):
        """compute_gravity_tree -> (acc, pot, (cell_interactions, particle_interactions))."""
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        acc = np.zeros((n, 3))
        pot = np.zeros(n)
        st = np.zeros(2, np.uint64)
        rc = self.lib.orc_tree_force(_p(pos, C.c_double), _p(mass, C.c_double), n, G, theta, eps,
                                     int(quadrupole), leaf_size, parallel_threshold,
                                     _p(acc, C.c_double), _p(pot, C.c_double),
                                     _p(st, C.c_uint64))
        if rc:
            raise RuntimeError(self.error())
        return acc, pot, (int(st[0]), int(st[1]))

    def direct_fp64(self, pos, mass, G=1.0, eps=0.025, idx=None):
        """FP64 direct summation for targets idx (all if None) -> (acc (m,3), pot (m,))."""
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        ia = None if idx is None else np.ascontiguousarray(idx, dtype=np.uint64)
        m = n if ia is None else ia.shape[0]
        acc = np.zeros((m, 3))
        pot = np.zeros(m)
        self.lib.orc_direct_fp64(_p(pos, C.c_double), _p(mass, C.c_double), n, _p(ia, C.c_uint64),
                                 m, G, eps, _p(acc, C.c_double), _p(pot, C.c_double))
        return acc, pot

    def pack_bodies(self, pos, mass, origin):
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        out = np.zeros((n, 4), np.float32)
        o = _f64(origin)
        self.lib.orc_pack_bodies(_p(pos, C.c_double), _p(mass, C.c_double), n, _p(o, C.c_double),
                                 _p(out, C.c_float))
        return out

    def direct_fp32(self, bodies, G=1.0, eps=0.025, idx=None):
        bodies = np.ascontiguousarray(bodies, dtype=np.float32)
        n = bodies.shape[0]
        ia = None if idx is None else np.ascontiguousarray(idx, dtype=np.uint64)
        m = n if ia is None else ia.shape[0]
        out = np.zeros((m, 4), np.float32)
        self.lib.orc_direct_fp32(_p(bodies, C.c_float), n, _p(ia, C.c_uint64), m, G, eps,
                                 _p(out, C.c_float))
        return out

    def leapfrog_group(self, pos, vel, mass, dt, steps, G=1.0, theta=0.75, eps=0.025,
                       group_size=32, leaf_size=8, pack=False):
        pos, vel, mass = _f64(pos).copy(), _f64(vel).copy(), _f64(mass)
        e = np.zeros(2)
        rc = self.lib.orc_leapfrog_group(_p(pos, C.c_double), _p(vel, C.c_double),
                                         _p(mass, C.c_double), mass.shape[0], G, theta, eps,
                                         group_size, leaf_size, int(pack), dt, steps,
                                         _p(e, C.c_double))
        if rc:
            raise RuntimeError(self.error())
        return pos, vel, e


class RefModel(C.Structure):
    _fields_ = [("G", C.c_double), ("disk_n", C.c_uint64), ("bulge_n", C.c_uint64),
                ("halo_n", C.c_uint64), ("disk_mass", C.c_double), ("disk_h", C.c_double),
                ("disk_z0", C.c_double), ("disk_rmax", C.c_double), ("disk_Q", C.c_double),
                ("disk_Q_radius", C.c_double), ("bulge_mass", C.c_double),
                ("bulge_a", C.c_double), ("bulge_rmax", C.c_double), ("halo_mass", C.c_double),
                ("halo_core", C.c_double), ("halo_cutoff", C.c_double),
                ("halo_rmax", C.c_double), ("vesc_fraction", C.c_double), ("seed", C.c_uint64),
                ("eps", C.c_double), ("theta", C.c_double)]


class Ref(_Common):
    """The reference itself (oracle/_ref/libgtref.so)."""

    def __init__(self, path=REF_SO):
        super().__init__(C.CDLL(str(path)), "ref_")
        L = self.lib
        V, D, U64, I = C.c_void_p, C.c_double, C.c_uint64, C.c_int
        pD, pF, pU32, pU64, pI = (C.POINTER(C.c_double), C.POINTER(C.c_float),
                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                  C.POINTER(C.c_int))
        L.ref_lists_build.restype = V
        L.ref_lists_build.argtypes = [V, D, D, D, I, I, I]
        L.ref_lists_eval.restype = None
        L.ref_lists_eval.argtypes = [V, D, D, I, pF]
        L.ref_group_force.restype = I
        L.ref_group_force.argtypes = [pD, pD, U64, D, D, D, I, I, I, I, I, pD, pD, V]
        L.ref_tree_force.restype = I
        L.ref_tree_force.argtypes = [pD, pD, U64, D, D, D, I, I, pD, pD, pU64]
        L.ref_direct_fp64.restype = None
        L.ref_direct_fp64.argtypes = [pD, pD, U64, D, D, pD, pD]
        L.ref_direct_fp32.restype = None
        L.ref_direct_fp32.argtypes = [pD, pD, U64, pD, D, D, pF, pF]
        L.ref_galaxy.restype = I
        L.ref_galaxy.argtypes = [C.POINTER(RefModel), pD, pD, pD, pI]
        L.ref_leapfrog_group.restype = I
        L.ref_leapfrog_group.argtypes = [pD, pD, pD, U64, D, D, D, I, I, I, D, I, pD]

    def lists(self, pos, mass, theta=0.75, group_size=32, leaf_size=8, pack=True,
              parallel_threshold=NO_PARALLEL, G=1.0, eps=0.025, quadrupole=True, evaluate=False):
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        L = self.lib
        th = L.ref_tree_build(_p(pos, C.c_double), _p(mass, C.c_double), n, leaf_size,
                              parallel_threshold)
        if not th:
            raise RuntimeError(self.error())
        try:
            nn = L.ref_tree_nnodes(th)
            nodes = np.zeros(nn, dtype=NODE_DTYPE)
            order = np.zeros(n, dtype=np.uint64)
            L.ref_tree_export(th, nodes.ctypes.data, _p(order, C.c_uint64))
            lh = L.ref_lists_build(th, G, theta, eps, int(quadrupole), group_size, int(pack))
            if not lh:
                raise RuntimeError(self.error())
            try:
                lists = self._export_lists(lh, n, nn)
                out = None
                if evaluate:
                    out = np.zeros((n, 4), np.float32)
                    L.ref_lists_eval(lh, G, eps, int(quadrupole), _p(out, C.c_float))
                return nodes, order, lists, out
            finally:
                L.ref_lists_free(lh)
        finally:
            L.ref_tree_free(th)

    def group_force(self, pos, mass, G=1.0, theta=0.75, eps=0.025, quadrupole=True,
                    group_size=32, leaf_size=8, pack=False, repeat=1):
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        acc = np.zeros((n, 3))
        pot = np.zeros(n)
        buf = np.zeros(5, np.float64)
        rc = self.lib.ref_group_force(_p(pos, C.c_double), _p(mass, C.c_double), n, G, theta, eps,
                                      int(quadrupole), group_size, leaf_size, int(pack), repeat,
                                      _p(acc, C.c_double), _p(pot, C.c_double), buf.ctypes.data)
        if rc:
            raise RuntimeError(self.error())
        ints = buf[3:].view(np.uint64)
        return acc, pot, dict(tree=buf[0], lists=buf[1], evaluate=buf[2],
                              cell_interactions=int(ints[0]), body_interactions=int(ints[1]))

    def tree_force(self, pos, mass, G=1.0, theta=0.75, eps=0.025, quadrupole=True, leaf_size=8):
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        acc = np.zeros((n, 3))
        pot = np.zeros(n)
        st = np.zeros(2, np.uint64)
        rc = self.lib.ref_tree_force(_p(pos, C.c_double), _p(mass, C.c_double), n, G, theta, eps,
                                     int(quadrupole), leaf_size, _p(acc, C.c_double),
                                     _p(pot, C.c_double), _p(st, C.c_uint64))
        if rc:
            raise RuntimeError(self.error())
        return acc, pot, (int(st[0]), int(st[1]))

    def direct_fp64(self, pos, mass, G=1.0, eps=0.025):
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        acc = np.zeros((n, 3))
        pot = np.zeros(n)
        self.lib.ref_direct_fp64(_p(pos, C.c_double), _p(mass, C.c_double), n, G, eps,
                                 _p(acc, C.c_double), _p(pot, C.c_double))
        return acc, pot

    def direct_fp32(self, pos, mass, origin, G=1.0, eps=0.025):
        pos, mass = _f64(pos), _f64(mass)
        n = mass.shape[0]
        bodies = np.zeros((n, 4), np.float32)
        out = np.zeros((n, 4), np.float32)
        o = _f64(origin)
        self.lib.ref_direct_fp32(_p(pos, C.c_double), _p(mass, C.c_double), n, _p(o, C.c_double),
                                 G, eps, _p(bodies, C.c_float), _p(out, C.c_float))
        return bodies, out

    def galaxy(self, n=None, seed=1, disk_n=None, bulge_n=None, halo_n=None, **kw):
        """make_hernquist_galaxy with the benchmark model unless fields are given."""
        m = RefModel(**reference_galaxy_model(n, seed, disk_n, bulge_n, halo_n, **kw))
        tot = m.disk_n + m.bulge_n + m.halo_n
        pos = np.zeros((tot, 3))
        vel = np.zeros((tot, 3))
        mass = np.zeros(tot)
        typ = np.zeros(tot, np.int32)
        rc = self.lib.ref_galaxy(C.byref(m), _p(pos, C.c_double), _p(vel, C.c_double),
                                 _p(mass, C.c_double), _p(typ, C.c_int))
        if rc:
            raise RuntimeError(self.error())
        return pos, vel, mass, typ

    def leapfrog_group(self, pos, vel, mass, dt, steps, G=1.0, theta=0.75, eps=0.025,
                       group_size=32, leaf_size=8, pack=False):
        pos, vel, mass = _f64(pos).copy(), _f64(vel).copy(), _f64(mass)
        e = np.zeros(2)
        rc = self.lib.ref_leapfrog_group(_p(pos, C.c_double), _p(vel, C.c_double),
                                         _p(mass, C.c_double), mass.shape[0], G, theta, eps,
                                         group_size, leaf_size, int(pack), dt, steps,
                                         _p(e, C.c_double))
        if rc:
            raise RuntimeError(self.error())
        return pos, vel, e


def reference_galaxy_model(n=None, seed=1, disk_n=None, bulge_n=None, halo_n=None, **kw):
    """The benchmark galaxy: disk 40% (M=1, h=1, z0=0.1), bulge 13% (M=0.33, a=0.2),
    halo the rest (M=5.8, core 1, cutoff 10); other fields at the reference's
    defaults (include/galactic_tides/hernquist_ics.h:55-77)."""
    if n is not None:
        disk_n = int(n * 40 // 100)
        bulge_n = int(n * 13 // 100)
        halo_n = int(n) - disk_n - bulge_n
    m = dict(G=1.0, disk_n=disk_n, bulge_n=bulge_n, halo_n=halo_n, disk_mass=1.0, disk_h=1.0,
             disk_z0=0.1, disk_rmax=10.0, disk_Q=1.5, disk_Q_radius=2.43, bulge_mass=0.33,
             bulge_a=0.2, bulge_rmax=4.0, halo_mass=5.8, halo_core=1.0, halo_cutoff=10.0,
             halo_rmax=30.0, vesc_fraction=0.95, seed=seed, eps=0.025, theta=0.75)
    m.update(kw)
    return m


def have_ref():
    return REF_SO.exists()


# ----------------------------------------------------------- test systems

def lopsided_sphere(n, seed):
    """A Hernquist sphere with 10% of the mass in two compact satellites: the
    shape of the reference tests' make_test_system (tests/test_gpu_kernels.cpp:29-47),
    drawn from numpy's PCG64 instead of mt19937_64."""
    rng = np.random.default_rng(seed)
    i = np.arange(n)
    centre = np.zeros((n, 3))
    a = np.ones(n)
    sat = i % 10 == 0
    centre[sat & (i % 20 == 0)] = (4.0, 0.0, 0.0)
    centre[sat & (i % 20 != 0)] = (-1.0, 3.0, 2.0)
    a[sat] = 0.1
    x = np.sqrt(rng.random(n) * 0.95)
    r = a * x / (1 - x)
    cz = 2 * rng.random(n) - 1
    ph = 2 * np.pi * rng.random(n)
    s = np.sqrt(1 - cz * cz)
    pos = centre + r[:, None] * np.stack([s * np.cos(ph), s * np.sin(ph), cz], axis=1)
    mass = np.full(n, 1.0 / n)
    return pos, mass


def coincident_system():
    """100 coincident bodies plus 50 spread ones (tests/test_gpu_kernels.cpp:276-288)."""
    pos = np.zeros((150, 3))
    pos[:100] = (1.0, 2.0, 3.0)
    k = np.arange(50, dtype=np.float64)
    pos[100:, 0] = k
    pos[100:, 1] = -k
    pos[100:, 2] = 0.5 * k
    return pos, np.ones(150)
