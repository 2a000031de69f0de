"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

``librmsd_oracle.so`` is the FP64 restatement in ``rmsd_oracle.c``;
``_ref/libcpptraj_rmsd_ref.so`` is cpptraj's own Frame RMSD code compiled from
its sources (present only where those sources were available at build time).
Only tests, ``__graft_entry__.smoke`` and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "librmsd_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libcpptraj_rmsd_ref.so")
# The reference's source tree (cpptraj's src/), used only to build _ref/;
# GBR_REFERENCE_SRC overrides the default location.
REF_SRC = os.environ.get("GBR_REFERENCE_SRC", "/root/reference/src")

FIT, NOFIT, QCP, DME = 0, 1, 2, 3
TRI, FULL = 0, 1

_lib = None
_ref = None


def build(with_ref: bool = True) -> None:
    """Compile the oracle (and, when the reference sources exist, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "-j8"], check=True)
    if with_ref and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "-j8", "ref"], check=True)


def _p(a):
    return ctypes.c_void_p(0) if a is None else a.ctypes.data_as(ctypes.c_void_p)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(with_ref=False)
        L = ctypes.CDLL(LIB)
        L.orc_allpairs.restype = ctypes.c_int
        L.orc_allpairs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                   ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                                   ctypes.c_int64, ctypes.c_int]
        L.orc_allpairs_f64.restype = ctypes.c_int
        L.orc_allpairs_f64.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        L.orc_pairs_f64.restype = ctypes.c_int
        L.orc_pairs_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_void_p, ctypes.c_int]
        L.orc_superpose_f64.restype = ctypes.c_int
        L.orc_superpose_f64.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.orc_cluster_centroids_f64.restype = ctypes.c_int
        L.orc_cluster_centroids_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int,
                                                ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_int64, ctypes.c_void_p, ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_grad_f64.restype = ctypes.c_int
        L.orc_grad_f64.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.orc_fd_f64.restype = ctypes.c_double
        L.orc_fd_f64.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_int]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_LIB)
        L.ref_allpairs.restype = ctypes.c_int
        L.ref_allpairs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                   ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        L.ref_write_cmatrix.restype = ctypes.c_int
        L.ref_write_cmatrix.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_int64, ctypes.c_int]
        L.ref_pairs_f64.restype = ctypes.c_int
        L.ref_pairs_f64.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_void_p]
        L.ref_superpose.restype = ctypes.c_int
        L.ref_superpose.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.ref_cluster_centroids.restype = ctypes.c_int
        L.ref_cluster_centroids.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int64, ctypes.c_void_p]
        _ref = L
    return _ref


def _dtype_code(x):
    if x.dtype == np.float64:
        return 1
    if x.dtype == np.float32:
        return 0
    raise TypeError("coordinates must be float32 or float64")


def n_out(n_ref, n_tgt, out_kind, row_begin=0, row_end=None):
    """Elements in rows [row_begin, row_end): TRI rows are reference frames,
    FULL rows are target frames (the slow index of the FULL layout)."""
    if out_kind == TRI:
        if row_end is None or row_end < 0:
            row_end = n_ref

        def cnt(i):
            return i * n_ref - (i * (i + 1)) // 2
        return cnt(row_end) - cnt(row_begin)
    if row_end is None or row_end < 0:
        row_end = n_tgt
    return (row_end - row_begin) * n_ref


def allpairs(ref, tgt=None, ref_mass=None, tgt_mass=None, mode=FIT, out_kind=None,
             row_begin=0, row_end=None, nthreads=0, use_reference_code=False):
    """All-pairs RMSD with rms2d semantics; returns the float32 output array."""
    ref = np.ascontiguousarray(ref)
    n_ref, n_atom = ref.shape[0], ref.shape[1]
    if tgt is not None:
        tgt = np.ascontiguousarray(tgt, dtype=ref.dtype)
    n_tgt = n_ref if tgt is None else tgt.shape[0]
    if out_kind is None:
        out_kind = TRI if tgt is None else FULL
    if tgt_mass is not None:
        tgt_mass = np.ascontiguousarray(tgt_mass, dtype=np.float64)
    if ref_mass is not None:
        ref_mass = np.ascontiguousarray(ref_mass, dtype=np.float64)
    elif tgt_mass is not None:
        ref_mass = tgt_mass
    if row_end is None:
        row_end = -1
    if use_reference_code:
        out = np.zeros(n_out(n_ref, n_tgt, out_kind), np.float32)
        rc = ref_lib().ref_allpairs(_p(ref), _p(tgt), _dtype_code(ref), n_ref, n_tgt, n_atom,
                                    _p(ref_mass), _p(tgt_mass), mode, out_kind, _p(out), nthreads)
    else:
        out = np.zeros(n_out(n_ref, n_tgt, out_kind, row_begin, row_end), np.float32)
        rc = lib().orc_allpairs(_p(ref), _p(tgt), _dtype_code(ref), n_ref, n_tgt, n_atom,
                                _p(ref_mass), _p(tgt_mass), mode, out_kind, _p(out),
                                row_begin, row_end, nthreads)
    if rc & 1:
        raise ValueError("oracle rejected arguments")
    return out


def allpairs_f64(ref, tgt=None, ref_mass=None, tgt_mass=None, mode=FIT, out_kind=None, nthreads=0):
    ref = np.ascontiguousarray(ref)
    n_ref, n_atom = ref.shape[0], ref.shape[1]
    if tgt is not None:
        tgt = np.ascontiguousarray(tgt, dtype=ref.dtype)
    n_tgt = n_ref if tgt is None else tgt.shape[0]
    if out_kind is None:
        out_kind = TRI if tgt is None else FULL
    if tgt_mass is not None:
        tgt_mass = np.ascontiguousarray(tgt_mass, dtype=np.float64)
    if ref_mass is None:
        ref_mass = tgt_mass
    else:
        ref_mass = np.ascontiguousarray(ref_mass, dtype=np.float64)
    out = np.zeros(n_out(n_ref, n_tgt, out_kind), np.float64)
    lib().orc_allpairs_f64(_p(ref), _p(tgt), _dtype_code(ref), n_ref, n_tgt, n_atom,
                           _p(ref_mass), _p(tgt_mass), mode, out_kind, _p(out), nthreads)
    return out


def pairs_f64(xyz, pi, pj, mass=None, mode=FIT, nthreads=0, use_reference_code=False):
    """RMSD for an explicit list of (ref=pi, tgt=pj) pairs, FP64."""
    xyz = np.ascontiguousarray(xyz)
    pi = np.ascontiguousarray(pi, dtype=np.int64)
    pj = np.ascontiguousarray(pj, dtype=np.int64)
    if mass is not None:
        mass = np.ascontiguousarray(mass, dtype=np.float64)
    out = np.zeros(len(pi), np.float64)
    if use_reference_code:
        ref_lib().ref_pairs_f64(_p(xyz), _dtype_code(xyz), xyz.shape[1], _p(mass), mode,
                                _p(pj), _p(pi), len(pi), _p(out))
    else:
        lib().orc_pairs_f64(_p(xyz), _dtype_code(xyz), xyz.shape[1], _p(mass), mode, _p(pi), _p(pj),
                            len(pi), _p(out), nthreads)
    return out


def tri_index(n, i, j):
    return n * i - ((i + 1) * i) // 2 + j - i - 1


def grad_f64(xyz, mass=None, g=None, nthreads=0):
    """Analytic FP64 gradient of L = sum_{i<j} g_ij RMSD_ij (xyz float32)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    if mass is not None:
        mass = np.ascontiguousarray(mass, dtype=np.float64)
    if g is not None:
        g = np.ascontiguousarray(g, dtype=np.float32)
    out = np.zeros(xyz.shape, np.float64)
    lib().orc_grad_f64(_p(xyz), xyz.shape[0], xyz.shape[1], _p(mass), _p(g), _p(out), nthreads)
    return out


def fd_f64(xyz, f, a, p, h=1e-3, mass=None, g=None, nthreads=0):
    """Central finite difference dL/dxyz[f, a, p] with step h (FP64 arithmetic)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    if mass is not None:
        mass = np.ascontiguousarray(mass, dtype=np.float64)
    if g is not None:
        g = np.ascontiguousarray(g, dtype=np.float32)
    return lib().orc_fd_f64(_p(xyz), xyz.shape[0], xyz.shape[1], _p(mass), _p(g), f, a, p, h, nthreads)


def ref_write_cmatrix(path, tri, frame_to_idx, sieve):
    """Write a pairwise cache with cpptraj's own Cmatrix_Binary writer (oracle/_ref)."""
    tri = np.ascontiguousarray(tri, dtype=np.float32)
    f2i = np.ascontiguousarray(frame_to_idx, dtype=np.int32)
    nrows = int((f2i >= 0).sum())
    rc = ref_lib().ref_write_cmatrix(path.encode(), _p(tri), _p(f2i), len(f2i), nrows, int(sieve))
    if rc != 0:
        raise RuntimeError("reference cmatrix writer failed")


def superpose_f64(ref, xyz, ref_mass=None, mass=None, mode=FIT, move=None, nthreads=0, use_reference_code=False):
    """Per-frame fit onto one reference frame (rms / align actions).  Returns
    (rmsd [F], rot [F,3,3], tgt_trans [F,3], ref_trans [3], moved [F,M,3] or
    None), all FP64.  ``move`` (FP64 [F, M, 3]) is copied, then moved."""
    ref = np.ascontiguousarray(ref)
    xyz = np.ascontiguousarray(xyz, dtype=ref.dtype)
    F, N = xyz.shape[0], xyz.shape[1]
    if mass is not None:
        mass = np.ascontiguousarray(mass, dtype=np.float64)
    if ref_mass is not None:
        ref_mass = np.ascontiguousarray(ref_mass, dtype=np.float64)
    rmsd = np.zeros(F)
    rot = np.zeros((F, 3, 3))
    tt = np.zeros((F, 3))
    rt = np.zeros(3)
    mv = None if move is None else np.array(move, dtype=np.float64, order="C", copy=True)
    nm = 0 if mv is None else mv.shape[1]
    if use_reference_code:
        ref_lib().ref_superpose(_p(ref), _p(xyz), _dtype_code(ref), F, N, _p(ref_mass), _p(mass), _p(rmsd), _p(rot),
                                _p(tt), _p(rt), _p(mv), nm)
    else:
        lib().orc_superpose_f64(_p(ref), _p(xyz), _dtype_code(ref), F, N, _p(ref_mass), _p(mass), mode, _p(rmsd),
                                _p(rot), _p(tt), _p(rt), _p(mv), nm, nthreads)
    return rmsd, rot, tt, rt, mv


def members_offsets(labels, n_cluster=None):
    """Cluster member lists in the reference's visiting order (increasing frame
    index within a cluster) from per-frame labels (-1 = noise, no cluster):
    (members int32, offsets int64 [n_cluster + 1])."""
    labels = np.asarray(labels)
    if n_cluster is None:
        n_cluster = int(labels.max()) + 1 if labels.size else 0
    members = [np.flatnonzero(labels == c) for c in range(n_cluster)]
    offsets = np.zeros(n_cluster + 1, np.int64)
    offsets[1:] = np.cumsum([len(m) for m in members])
    flat = np.concatenate(members) if members else np.zeros(0)
    return flat.astype(np.int32), offsets


def cluster_centroids_f64(xyz, members, offsets, mass=None, mode=FIT, nthreads=0, use_reference_code=False):
    """Cluster centroids (Metric_RMS::CalculateCentroid): [n_cluster, N, 3]
    FP64.  members / offsets as returned by members_offsets."""
    xyz = np.ascontiguousarray(xyz)
    F, N = xyz.shape[0], xyz.shape[1]
    members = np.ascontiguousarray(members, dtype=np.int32)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    nc = len(offsets) - 1
    if mass is not None:
        mass = np.ascontiguousarray(mass, dtype=np.float64)
    out = np.zeros((nc, N, 3))
    if use_reference_code:
        rc = ref_lib().ref_cluster_centroids(_p(xyz), _dtype_code(xyz), F, N, _p(mass), mode, _p(members),
                                             _p(offsets), nc, _p(out))
    else:
        rc = lib().orc_cluster_centroids_f64(_p(xyz), _dtype_code(xyz), F, N, _p(mass), mode, _p(members),
                                             _p(offsets), nc, _p(out), nthreads)
    if rc != 0:
        raise ValueError("cluster centroids: error %d" % rc)
    return out
