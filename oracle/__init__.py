"""CPU oracle for the Voxel Cores hot path -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline / reference
legs of ``bench.py`` may import this package, and only as the checker or as
the timed CPU baseline; the product path never routes through it.

Two libraries are loaded through ctypes:

* ``liboracle.so`` -- the project's restatement (``vc_oracle.cpp``) of the
  reference's site sweep, the nearest-site relation, the lattice Voronoi
  inside-extraction with lambda measures, ``cellcomplex::finalize``,
  ``CellComplexThinning::prune`` / ``remainingCC``,
  ``util::computeEulerChar``, ``nClosedComponents``, the ``.sof`` / ``.sog``
  octree readers and the ``.ply`` / ``.r`` / ``.ma`` writers.  Builds on any
  host (``make oracle``).
* ``_ref/libvcref.so`` -- the reference's OWN sources (ccthin.cpp,
  cellcomplex.cpp, geomalgo.cpp, octree.cpp, spaceinfo.cpp, surfacing.cpp,
  and writeToDotma cut out of exporters.cpp) compiled against the API shim in
  ``shim/`` (``make ref``).  Only buildable where the reference tree exists;
  used to pin the restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None
# The reference's source tree, named by the build recipe or the environment
# (VOXEL_MA_REFERENCE); no default: hosts without the tree build no _ref.
_REFERENCE_TREE = os.environ.get("VOXEL_MA_REFERENCE", "")

c_i64 = ctypes.c_longlong
c_vp = ctypes.c_void_p


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(c_vp)


def build(reference: bool = True, tree: Optional[str] = None) -> None:
    """Compile liboracle.so, and the reference library when the reference's
    tree (`tree`, else $VOXEL_MA_REFERENCE) exists."""
    global _REFERENCE_TREE
    if tree:
        _REFERENCE_TREE = tree
    subprocess.run(["make", "-s", "-C", _HERE, "oracle"], check=True)
    if reference and reference_tree_present():
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REFERENCE={_REFERENCE_TREE}"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build(reference=False)
        L = ctypes.CDLL(path)
        L.vco_extract_sites.restype = c_i64
        L.vco_extract_sites.argtypes = [c_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_vp, c_vp, c_i64]
        L.vco_ft_bruteforce.argtypes = [ctypes.c_int] * 3 + [c_i64, c_vp, c_vp, c_vp]
        L.vco_ft.argtypes = [ctypes.c_int] * 3 + [c_i64, c_vp, c_vp, c_vp, ctypes.c_int]
        L.vco_lattice_vd.restype = c_vp
        L.vco_lattice_vd.argtypes = [c_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_vp, c_vp]
        L.vco_vd_sizes.argtypes = [c_vp] * 6
        L.vco_lattice_vd_counts.argtypes = [c_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_vp, c_vp, c_vp]
        L.vco_vd_get.argtypes = [c_vp] * 9
        L.vco_vd_radius.argtypes = [c_vp, c_vp]
        L.vco_vd_free.argtypes = [c_vp]
        L.vco_finalize.restype = c_i64
        L.vco_finalize.argtypes = [c_i64, c_i64, c_vp, c_i64, c_vp] + [c_vp] * 6
        L.vco_thin.restype = ctypes.c_int
        L.vco_thin.argtypes = [c_i64, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, ctypes.c_float, ctypes.c_float,
                               c_vp, c_vp, c_vp, c_vp, c_vp]
        L.vco_remaining.argtypes = [c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp,
                                    c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]
        L.vco_euler.argtypes = [c_i64, c_i64, c_vp, c_i64, c_vp, c_vp]
        L.vco_sof_decode.restype = ctypes.c_int
        L.vco_sof_decode.argtypes = [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]
        L.vco_sog_decode.restype = ctypes.c_int
        L.vco_sog_decode.argtypes = [c_vp, c_i64, c_vp, c_vp, c_vp, c_vp]
        L.vco_closed_components.restype = c_i64
        L.vco_closed_components.argtypes = [c_i64, c_i64, c_vp, c_i64, c_vp]
        for name, args in (("vco_write_dotma", [ctypes.c_char_p, c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]),
                           ("vco_write_radii", [ctypes.c_char_p, c_vp, c_vp, c_i64]),
                           ("vco_write_ply", [ctypes.c_char_p, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64])):
            getattr(L, name).restype = ctypes.c_int
            getattr(L, name).argtypes = args
        L.vco_dotma_edges.restype = c_i64
        L.vco_dotma_edges.argtypes = [c_vp, c_i64, c_vp, c_i64, c_vp]
        _LIB = L
    return _LIB


def ref_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libvcref.so"))


def reference_tree_present() -> bool:
    """Whether the reference's source tree is on this host (the recipe builds from it)."""
    return bool(_REFERENCE_TREE) and os.path.isdir(os.path.join(_REFERENCE_TREE, "src"))


def ref():
    """The reference's own compiled sources (raises if not built here)."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libvcref.so")
        if not os.path.exists(path):
            raise FileNotFoundError("oracle/_ref/libvcref.so is not built (needs the reference tree)")
        R = ctypes.CDLL(path)
        R.vcref_extract_sites.restype = c_i64
        R.vcref_extract_sites.argtypes = [c_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_vp, c_i64]
        R.vcref_cc_create.restype = c_vp
        R.vcref_cc_create.argtypes = [ctypes.c_int, c_vp, ctypes.c_int, c_vp, ctypes.c_int, c_vp]
        R.vcref_cc_destroy.argtypes = [c_vp]
        R.vcref_cc_num_edges.restype = ctypes.c_int
        R.vcref_cc_num_edges.argtypes = [c_vp]
        R.vcref_cc_get_edges.argtypes = [c_vp, c_vp]
        R.vcref_cc_get_face_edges.argtypes = [c_vp, c_vp]
        R.vcref_cc_adj_size.restype = c_i64
        R.vcref_cc_adj_size.argtypes = [c_vp, ctypes.c_int]
        R.vcref_cc_get_adj.argtypes = [c_vp, ctypes.c_int, c_vp, c_vp]
        R.vcref_sof_write.restype = ctypes.c_int
        R.vcref_write_dotma.restype = ctypes.c_int
        R.vcref_write_dotma.argtypes = [ctypes.c_char_p, c_vp, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64]
        R.vcref_dotma_edges.restype = c_i64
        R.vcref_dotma_edges.argtypes = [c_vp, c_i64, c_vp, c_i64, c_vp]
        R.vcref_sof_write.argtypes = [c_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p]
        R.vcref_sof_occupancy.restype = ctypes.c_int
        R.vcref_sof_occupancy.argtypes = [ctypes.c_char_p, c_vp]
        R.vcref_sof_sites.restype = c_i64
        R.vcref_sof_sites.argtypes = [ctypes.c_char_p, c_vp, c_i64]
        R.vcref_closed_components.restype = ctypes.c_int
        R.vcref_closed_components.argtypes = [ctypes.c_int, c_vp, ctypes.c_int, c_vp, ctypes.c_int, c_vp]
        R.vcref_thin.restype = ctypes.c_int
        R.vcref_thin.argtypes = [c_vp, c_vp, c_vp, c_vp, ctypes.c_float, ctypes.c_float, c_vp, c_vp, c_vp, c_vp]
        R.vcref_remaining_sizes.argtypes = [c_vp, c_vp, c_vp, c_vp]
        R.vcref_remaining_get.argtypes = [c_vp, c_vp, c_vp, c_vp]
        R.vcref_euler.argtypes = [ctypes.c_int, c_vp, ctypes.c_int, c_vp, ctypes.c_int, c_vp, c_vp]
        R.vcref_simple_triangulate.restype = ctypes.c_int
        R.vcref_simple_triangulate.argtypes = [ctypes.c_int, c_vp, c_vp]
        _REF = R
    return _REF


# --------------------------------------------------------------------------
# restatement (liboracle.so)

def extract_sites(occ: np.ndarray):
    """Sites of a (X,Y,Z) uint8 volume: (xyz float32 [n,3], lattice index int64 [n])."""
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    X, Y, Z = occ.shape
    L = lib()
    n = L.vco_extract_sites(_ptr(occ), X, Y, Z, None, None, 0)
    xyz = np.zeros((n, 3), np.float32)
    li = np.zeros(n, np.int64)
    L.vco_extract_sites(_ptr(occ), X, Y, Z, _ptr(xyz), _ptr(li), n)
    return xyz, li


def ft(shape, site_lattice_idx: np.ndarray, brute: bool = False, threads: int = 1):
    """Exact nearest-site transform on the corner lattice: (d2 int32, id int32), shape (X+1,Y+1,Z+1)."""
    X, Y, Z = shape
    li = np.ascontiguousarray(site_lattice_idx, dtype=np.int64)
    n = (X + 1) * (Y + 1) * (Z + 1)
    d2 = np.zeros(n, np.int32)
    ids = np.zeros(n, np.int32)
    if brute:
        lib().vco_ft_bruteforce(X, Y, Z, len(li), _ptr(li), _ptr(d2), _ptr(ids))
    else:
        lib().vco_ft(X, Y, Z, len(li), _ptr(li), _ptr(d2), _ptr(ids), threads)
    return d2.reshape(X + 1, Y + 1, Z + 1), ids.reshape(X + 1, Y + 1, Z + 1)


def lattice_vd_counts(occ: np.ndarray, ft_id: np.ndarray) -> dict:
    """The sizes lattice_vd would give (nv, ne, nt, nface) and its inside size, counted without building the
    complex (vco_lattice_vd_counts): for volumes whose complex does not fit in host memory."""
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    ft_id = np.ascontiguousarray(ft_id, dtype=np.int32)
    X, Y, Z = occ.shape
    sizes = np.zeros(4, np.int64)
    isz = ctypes.c_float()
    lib().vco_lattice_vd_counts(_ptr(occ), X, Y, Z, _ptr(ft_id), _ptr(sizes), ctypes.byref(isz))
    return dict(nv=int(sizes[0]), ne=int(sizes[1]), nt=int(sizes[2]), nface=int(sizes[3]), inside_size=float(isz.value))


def lattice_vd(occ: np.ndarray, ft_id: np.ndarray, site_xyz: np.ndarray) -> dict:
    """Inside lattice Voronoi complex with lambda measures (see vc_oracle.h)."""
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    ft_id = np.ascontiguousarray(ft_id, dtype=np.int32)
    sx = np.ascontiguousarray(site_xyz, dtype=np.float32)
    X, Y, Z = occ.shape
    L = lib()
    h = L.vco_lattice_vd(_ptr(occ), X, Y, Z, _ptr(ft_id), _ptr(sx))
    nv, ne, nt, nf = c_i64(), c_i64(), c_i64(), c_i64()
    isz = ctypes.c_float()
    L.vco_vd_sizes(h, ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(nt), ctypes.byref(nf), ctypes.byref(isz))
    out = dict(
        vts=np.zeros((nv.value, 3), np.float32), edges=np.zeros((ne.value, 2), np.int32),
        tris=np.zeros((nt.value, 3), np.int32), vm=np.zeros(nv.value, np.float32),
        em=np.zeros(ne.value, np.float32), fm=np.zeros(nt.value, np.float32),
        tri_face=np.zeros(nt.value, np.int32), face_sites=np.zeros((nf.value, 2), np.int32))
    L.vco_vd_get(h, *[_ptr(out[k]) for k in ("vts", "edges", "tris", "vm", "em", "fm", "tri_face", "face_sites")])
    out["radius"] = np.zeros(nv.value, np.float32)
    L.vco_vd_radius(h, _ptr(out["radius"]))
    L.vco_vd_free(h)
    out["inside_size"] = float(isz.value)
    return out


def finalize(nv: int, edges: np.ndarray, tris: np.ndarray) -> dict:
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    L = lib()
    ne = L.vco_finalize(nv, len(edges), _ptr(edges), len(tris), _ptr(tris), None, None, None, None, None, None)
    o = dict(edges=np.zeros((ne, 2), np.int32), tri_edges=np.zeros((len(tris), 3), np.int32),
             ve_off=np.zeros(nv + 1, np.int32), ve_ids=np.zeros(2 * ne, np.int32),
             ef_off=np.zeros(ne + 1, np.int32), ef_ids=np.zeros(3 * len(tris), np.int32))
    L.vco_finalize(nv, len(edges), _ptr(edges), len(tris), _ptr(tris), *[_ptr(o[k]) for k in
                   ("edges", "tri_edges", "ve_off", "ve_ids", "ef_off", "ef_ids")])
    return o


def finalize_edges(nv: int, edges: np.ndarray, tris: np.ndarray) -> np.ndarray:
    """The finalized edge list only (no adjacency lists): what the remaining
    complex needs, at a fraction of finalize()'s memory."""
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    cap = np.zeros((len(edges) + 3 * len(tris), 2), np.int32)  # upper bound of the finalized edges
    ne = lib().vco_finalize(nv, len(edges), _ptr(edges), len(tris), _ptr(tris), _ptr(cap), None, None, None, None,
                            None)
    out = cap[:ne].copy()
    del cap
    return out


def thin(nv: int, edges: np.ndarray, tris: np.ndarray, em_fin: np.ndarray, fm: np.ndarray, f_t: float, l_t: float):
    """FIFO prune; em_fin indexed by FINALIZED edge id.  Returns dict of flags + stats."""
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    em_fin = np.ascontiguousarray(em_fin, dtype=np.float32)
    fm = np.ascontiguousarray(fm, dtype=np.float32)
    ne = len(em_fin)
    kv, ke, kf, re = (np.zeros(nv, np.uint8), np.zeros(ne, np.uint8), np.zeros(len(tris), np.uint8),
                      np.zeros(ne, np.uint8))
    st = np.zeros(4, np.int64)
    rc = lib().vco_thin(nv, len(edges), _ptr(edges), len(tris), _ptr(tris), _ptr(em_fin), _ptr(fm),
                        ctypes.c_float(f_t), ctypes.c_float(l_t), _ptr(kv), _ptr(ke), _ptr(kf), _ptr(re), _ptr(st))
    return dict(rc=rc, keep_v=kv, keep_e=ke, keep_f=kf, removed_e=re,
                stats=dict(pushes=int(st[0]), processed=int(st[1]), skipped=int(st[2]), generations=int(st[3])))


def closed_components(nv: int, edges: np.ndarray, tris: np.ndarray) -> int:
    """nClosedComponents (highlevelalgo.cpp:993-1020) restated."""
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    return int(lib().vco_closed_components(nv, len(edges), _ptr(edges), len(tris), _ptr(tris)))


def sof_decode(data: bytes, sog: bool = False):
    """A .sof (or, with sog, .sog) octree file decoded as the reference reads
    it: (occupancy of the (R+1)^3 voxels, the octree sites in pre-order);
    None when malformed."""
    fn = lib().vco_sog_decode if sog else lib().vco_sof_decode
    buf = np.frombuffer(data, dtype=np.uint8)
    size, ns = ctypes.c_int(), ctypes.c_longlong()
    if fn(_ptr(buf), len(buf), ctypes.byref(size), None, None, ctypes.byref(ns)) != 0:
        return None
    n = size.value
    occ = np.zeros((n, n, n), np.uint8)
    sites = np.zeros((ns.value, 3), np.float32)
    fn(_ptr(buf), len(buf), ctypes.byref(size), _ptr(occ), _ptr(sites), ctypes.byref(ns))
    return occ, sites


def ref_sof_write(occ: np.ndarray, path: str) -> None:
    """The reference's octree of a dense occupancy volume, written as .sof."""
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    X, Y, Z = occ.shape
    assert ref().vcref_sof_write(_ptr(occ), X, Y, Z, path.encode()) == 0


def ref_sof_read(path: str):
    """The reference's reading of a .sof file: (occupancy, octree sites)."""
    n = ref().vcref_sof_occupancy(path.encode(), None)
    occ = np.zeros((n, n, n), np.uint8)
    ref().vcref_sof_occupancy(path.encode(), _ptr(occ))
    ns = ref().vcref_sof_sites(path.encode(), None, 0)
    sites = np.zeros((ns, 3), np.float32)
    ref().vcref_sof_sites(path.encode(), _ptr(sites), ns)
    return occ, sites


def ref_closed_components(vts, edges, tris) -> int:
    """The reference's own thinning, remainingCC() and compute_conn_cmpnts()."""
    vts = np.ascontiguousarray(vts, dtype=np.float32).reshape(-1, 3)
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    return int(ref().vcref_closed_components(len(vts), _ptr(vts), len(edges), _ptr(edges), len(tris), _ptr(tris)))


def remaining(vts, edges_fin, tris, keep_v, keep_e, keep_f):
    vts = np.ascontiguousarray(vts, dtype=np.float32).reshape(-1, 3)
    edges_fin = np.ascontiguousarray(edges_fin, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    kv, ke, kf = (np.ascontiguousarray(x, dtype=np.uint8) for x in (keep_v, keep_e, keep_f))
    nv, ne, nt = c_i64(), c_i64(), c_i64()
    L = lib()
    args = [len(vts), _ptr(vts), len(edges_fin), _ptr(edges_fin), len(tris), _ptr(tris), _ptr(kv), _ptr(ke),
            _ptr(kf), ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(nt)]
    L.vco_remaining(*args, None, None, None)
    ov, oe, ot = (np.zeros((nv.value, 3), np.float32), np.zeros((ne.value, 2), np.int32),
                  np.zeros((nt.value, 3), np.int32))
    L.vco_remaining(*args, _ptr(ov), _ptr(oe), _ptr(ot))
    return ov, oe, ot


def euler(nv: int, edges, tris):
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    out = np.zeros(5, np.int64)
    lib().vco_euler(nv, len(edges), _ptr(edges), len(tris), _ptr(tris), _ptr(out))
    return dict(V=int(out[0]), E=int(out[1]), F=int(out[2]), C=int(out[3]), euler=int(out[4]))


def run_plain(occ: np.ndarray, t: float = 0.04, threads: int = 1) -> dict:
    """The whole CPU path on one volume: sites, FT, lattice VD + measures, thin, remaining."""
    xyz, li = extract_sites(occ)
    d2, ids = ft(occ.shape, li, threads=threads)
    vd = lattice_vd(occ, ids, xyz)
    fin = dict(edges=finalize_edges(len(vd["vts"]), vd["edges"], vd["tris"]))
    em_fin = np.zeros(len(fin["edges"]), np.float32)
    em_fin[: len(vd["em"])] = vd["em"]
    thresh = float(np.float32(np.float64(vd["inside_size"]) * t))
    th = thin(len(vd["vts"]), vd["edges"], vd["tris"], em_fin, vd["fm"], thresh, thresh)
    rv, re_, rt = remaining(vd["vts"], fin["edges"], vd["tris"], th["keep_v"], th["keep_e"], th["keep_f"])
    return dict(sites=xyz, site_lattice=li, d2=d2, ids=ids, vd=vd, fin=fin, thresh=thresh, thin=th,
                rem_vts=rv, rem_edges=re_, rem_tris=rt)


# --------------------------------------------------------------------------
# the reference's own compiled sources (_ref/libvcref.so)

def ref_extract_sites(occ: np.ndarray) -> np.ndarray:
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    X, Y, Z = occ.shape
    R = ref()
    n = R.vcref_extract_sites(_ptr(occ), X, Y, Z, None, 0)
    out = np.zeros((n, 3), np.float32)
    R.vcref_extract_sites(_ptr(occ), X, Y, Z, _ptr(out), n)
    return out


class RefComplex:
    """A finalized reference ``cellcomplex`` with its ``CellComplexThinning``."""

    def __init__(self, vts, edges, tris):
        self.vts = np.ascontiguousarray(vts, dtype=np.float32).reshape(-1, 3)
        edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
        tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
        self.nt = len(tris)
        self.R = ref()
        self.h = self.R.vcref_cc_create(len(self.vts), _ptr(self.vts), len(edges), _ptr(edges), len(tris), _ptr(tris))
        self.ne = self.R.vcref_cc_num_edges(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.R.vcref_cc_destroy(self.h)
            self.h = None

    def edges(self):
        o = np.zeros((self.ne, 2), np.int32)
        self.R.vcref_cc_get_edges(self.h, _ptr(o))
        return o

    def tri_edges(self):
        o = np.zeros((self.nt, 3), np.int32)
        self.R.vcref_cc_get_face_edges(self.h, _ptr(o))
        return o

    def adjacency(self, which: int):
        n = len(self.vts) if which == 0 else self.ne
        offs = np.zeros(n + 1, np.int32)
        ids = np.zeros(self.R.vcref_cc_adj_size(self.h, which), np.int32)
        self.R.vcref_cc_get_adj(self.h, which, _ptr(offs), _ptr(ids))
        return offs, ids

    def thin(self, vm, em_fin, fm, f_t, l_t):
        vm, em_fin, fm = (np.ascontiguousarray(x, dtype=np.float32) for x in (vm, em_fin, fm))
        kv, ke, kf, re = (np.zeros(len(self.vts), np.uint8), np.zeros(self.ne, np.uint8),
                          np.zeros(self.nt, np.uint8), np.zeros(self.ne, np.uint8))
        self.R.vcref_thin(self.h, _ptr(vm), _ptr(em_fin), _ptr(fm), ctypes.c_float(f_t), ctypes.c_float(l_t),
                          _ptr(kv), _ptr(ke), _ptr(kf), _ptr(re))
        return dict(keep_v=kv, keep_e=ke, keep_f=kf, removed_e=re)

    def remaining(self):
        nv, ne, nt = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.R.vcref_remaining_sizes(self.h, ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(nt))
        ov, oe, ot = (np.zeros((nv.value, 3), np.float32), np.zeros((ne.value, 2), np.int32),
                      np.zeros((nt.value, 3), np.int32))
        self.R.vcref_remaining_get(self.h, _ptr(ov), _ptr(oe), _ptr(ot))
        return ov, oe, ot


def ref_euler(vts, edges, tris):
    vts = np.ascontiguousarray(vts, dtype=np.float32).reshape(-1, 3)
    edges = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
    out = np.zeros(5, np.int32)
    ref().vcref_euler(len(vts), _ptr(vts), len(edges), _ptr(edges), len(tris), _ptr(tris), _ptr(out))
    return dict(V=int(out[0]), E=int(out[1]), F=int(out[2]), C=int(out[3]), euler=int(out[4]))


# ---- output formats (highlevelalgo.cpp:855-955) ------------------------------

def _c(a, dtype, cols):
    a = np.ascontiguousarray(np.asarray(a, dtype).reshape(-1, cols) if cols else np.asarray(a, dtype).ravel())
    return a, _ptr(a)


def write_dotma(path: str, vts, radii, edges, tris) -> None:
    """writeToDotma (exporters.cpp:244-287), restated on std::ofstream."""
    (v, pv), (r, pr), (e, pe), (t, pt) = (_c(vts, np.float32, 3), _c(radii, np.float32, 0),
                                          _c(edges, np.int32, 2), _c(tris, np.int32, 3))
    assert lib().vco_write_dotma(os.fsencode(path), pv, pr, len(v), pe, len(e), pt, len(t)) == 0


def write_radii(path: str, vts, radii) -> None:
    """writeRadiiToFile (exporters.cpp:478-552) for remaining vertices, identity matrix."""
    (v, pv), (r, pr) = _c(vts, np.float32, 3), _c(radii, np.float32, 0)
    assert lib().vco_write_radii(os.fsencode(path), pv, pr, len(v)) == 0


def write_ply(path: str, vts, edges, tris) -> None:
    """ply::PLYWriter::write (plyall.cpp:98-171) with the ply library's ASCII writer."""
    (v, pv), (e, pe), (t, pt) = _c(vts, np.float32, 3), _c(edges, np.int32, 2), _c(tris, np.int32, 3)
    assert lib().vco_write_ply(os.fsencode(path), pv, len(v), pe, len(e), pt, len(t)) == 0


def _edges_via(fn, edges, tris):
    (e, pe), (t, pt) = _c(edges, np.int32, 2), _c(tris, np.int32, 3)
    n = fn(pe, len(e), pt, len(t), None)
    out = np.zeros((n, 2), np.int32)
    fn(pe, len(e), pt, len(t), _ptr(out))
    return out


def dotma_edges(edges, tris) -> np.ndarray:
    """The .ma edge list of highlevelalgo.cpp:911-945 (remaining edges, then the
    triangles' edges in the order of an unordered_set with ivec2Hash)."""
    return _edges_via(lib().vco_dotma_edges, edges, tris)


def ref_write_dotma(path: str, vts, radii, edges, tris) -> None:
    """The reference's own writeToDotma."""
    (v, pv), (r, pr), (e, pe), (t, pt) = (_c(vts, np.float32, 3), _c(radii, np.float32, 0),
                                          _c(edges, np.int32, 2), _c(tris, np.int32, 3))
    assert ref().vcref_write_dotma(os.fsencode(path), pv, pr, len(v), pe, len(e), pt, len(t)) == 0


def ref_dotma_edges(edges, tris) -> np.ndarray:
    """The .ma edge assembly on the reference's own ivec2 / ivec2Hash."""
    return _edges_via(ref().vcref_dotma_edges, edges, tris)


# ---- MRC density maps (readMRC, importers.cpp:45-60) --------------------------

_MRC_DTYPES = {0: "i1", 1: "i2", 2: "f4", 6: "u2", 12: "f2"}


def mrc_decode(data: bytes):
    """The occupancy (value > 0) of an .mrc file's map, x-major and z fastest,
    or None when malformed.  A restatement of the public MRC2014 layout (Tao
    Ju's reader, which the reference calls, is not in its tree): header words
    0-2 column / row / section counts, 3 the mode, 16-18 the axes of columns,
    rows and sections, 23 the extended-header bytes; bytes 212-213 the
    machine stamp; values after the header, columns fastest."""
    b = np.frombuffer(data, np.uint8)
    if len(b) < 1024:
        return None
    s0, s1 = int(b[212]), int(b[213])
    big = s0 == 0x11 and s1 == 0x11
    words = {e: np.frombuffer(data[:1024], e + "i4") for e in ("<", ">")}
    if not (s0 == 0x44 and s1 in (0x44, 0x41)) and not big:
        big = int(words["<"][3]) not in _MRC_DTYPES and int(words[">"][3]) in _MRC_DTYPES
    w = words[">" if big else "<"]
    n = [int(w[0]), int(w[1]), int(w[2])]
    mode, nsym = int(w[3]), int(w[23])
    if min(n) <= 0 or max(n) > 32766 or mode not in _MRC_DTYPES or nsym < 0:
        return None
    ax = [int(w[16]) - 1, int(w[17]) - 1, int(w[18]) - 1]
    if sorted(ax) != [0, 1, 2]:
        ax = [0, 1, 2]
    dt = np.dtype(_MRC_DTYPES[mode]).newbyteorder(">" if big else "<")
    off = 1024 + nsym
    cnt = n[0] * n[1] * n[2]
    if len(b) < off + cnt * dt.itemsize:
        return None
    vals = np.frombuffer(data, dt, count=cnt, offset=off).reshape(n[2], n[1], n[0])  # sections, rows, columns
    # array axis k of vals runs along volume axis ax[2 - k]; order them x, y, z
    inv = [0, 0, 0]
    for k in range(3):
        inv[ax[2 - k]] = k
    return np.ascontiguousarray((vals > 0).transpose(inv)).astype(np.uint8)
