"""ctypes binding of libgbrmsd.so (the C ABI declared in include/gbrmsd.h).

The functions here take numpy arrays or torch tensors (host or CUDA) and call
the library directly; no computation happens in Python.  If the shared
library is missing the import of a function raises -- there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbrmsd.so")

GBR_OK = 0
GBR_F32, GBR_F64 = 0, 1
FIT, NOFIT, DME = 0, 1, 2
TRI, FULL = 0, 1
PREC_FP32, PREC_TC, PREC_FP64 = 0, 1, 2
OPT_TAU, OPT_MAX_REFS, OPT_TOL, OPT_TIMING, OPT_TC_PIPELINE, OPT_HOST_OUT, OPT_INPUT_OVERLAP = 0, 1, 2, 3, 4, 5, 6
OPT_BAND_FLOATS = 7
#: The library's default tensor-core kernel shape (pairs of SMs).
TC_PIPELINE_DEFAULT = -1  # automatic: deep stages from 1,280 atoms, wide chunks below 768, shallow between

PRECISIONS = {"fp32": PREC_FP32, "tc": PREC_TC, "fp64": PREC_FP64}
MODES = {"fit": FIT, "nofit": NOFIT, "dme": DME}

#: Every symbol include/gbrmsd.h declares.
EXPORTED = ("gbr_create", "gbr_destroy", "gbr_last_error", "gbr_allpairs", "gbr_output_count",
            "gbr_allpairs_batched", "gbr_rmsd_backward", "gbr_get_stats", "gbr_set_option", "gbr_set_stream",
            "gbr_write_cmatrix", "gbr_superpose", "gbr_cluster_centroids",
            "gbr_allpairs_fp64_static", "gbr_selftest_bounded_wait", "gbr_allpairs_stream", "gbr_row_bands")

#: C type of gbr_band_sink: (user, row_begin, row_end, values, count) -> int.
BAND_SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                             ctypes.POINTER(ctypes.c_float), ctypes.c_int64)


class GbrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbrmsd error {code}: {msg}")
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("pairs", ctypes.c_int64), ("pairs_fixed", ctypes.c_int64), ("n_refs", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("kernel_launches", ctypes.c_int32),
                ("ms_prep", ctypes.c_double), ("ms_pairs", ctypes.c_double), ("ms_fixup", ctypes.c_double),
                ("ms_total", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_lock = threading.Lock()


def load():
    """Load libgbrmsd.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built; run `python -m cpptraj_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, i32, ci, cd = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int, ctypes.c_double
        L.gbr_create.restype = vp
        L.gbr_create.argtypes = [ci]
        L.gbr_destroy.restype = None
        L.gbr_destroy.argtypes = [vp]
        L.gbr_last_error.restype = ctypes.c_char_p
        L.gbr_last_error.argtypes = [vp]
        L.gbr_allpairs.restype = ci
        L.gbr_allpairs.argtypes = [vp, vp, vp, ci, i64, i64, i32, vp, vp, ci, ci, ci, vp, i64, i64]
        L.gbr_output_count.restype = i64
        L.gbr_output_count.argtypes = [i64, i64, ci, i64, i64]
        L.gbr_allpairs_batched.restype = ci
        L.gbr_allpairs_batched.argtypes = [vp, i32, vp, vp, vp, vp, ci, ci, vp]
        L.gbr_rmsd_backward.restype = ci
        L.gbr_rmsd_backward.argtypes = [vp, vp, i64, i32, vp, vp, vp, vp]
        L.gbr_get_stats.restype = ci
        L.gbr_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.gbr_set_option.restype = ci
        L.gbr_set_option.argtypes = [vp, ci, cd]
        L.gbr_set_stream.restype = ci
        L.gbr_set_stream.argtypes = [vp, vp]
        L.gbr_write_cmatrix.restype = ci
        L.gbr_write_cmatrix.argtypes = [vp, ctypes.c_char_p, vp, ci, i64, i32, vp, ci, ci, vp, i64, i64]
        L.gbr_superpose.restype = ci
        L.gbr_superpose.argtypes = [vp, vp, vp, ci, i64, i32, vp, vp, ci, vp, vp, vp, vp, vp, i32]
        L.gbr_cluster_centroids.restype = ci
        L.gbr_cluster_centroids.argtypes = [vp, vp, ci, i64, i32, vp, ci, vp, vp, i64, vp]
        L.gbr_allpairs_fp64_static.restype = ci
        L.gbr_allpairs_fp64_static.argtypes = [vp, ci, i64, i32, vp, ci, vp, vp]
        L.gbr_allpairs_stream.restype = ci
        L.gbr_allpairs_stream.argtypes = [vp, vp, ci, i64, i32, vp, ci, ci, i64, BAND_SINK, vp]
        L.gbr_row_bands.restype = i64
        L.gbr_row_bands.argtypes = [i64, i64, i32, vp, i64]
        L.gbr_selftest_bounded_wait.restype = ci
        L.gbr_selftest_bounded_wait.argtypes = [vp, i64, vp, vp]
        _lib = L
        return L


def _ptr(x):
    """Raw pointer of a numpy array / torch tensor (or None)."""
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
        return x.ctypes.data
    # torch tensor
    if not x.is_contiguous():
        raise ValueError("tensors must be contiguous")
    return x.data_ptr()


def _dtype_code(x):
    dt = str(x.dtype)
    if dt.endswith("float32"):
        return GBR_F32
    if dt.endswith("float64"):
        return GBR_F64
    raise TypeError(f"coordinates must be float32 or float64, got {dt}")


def _shape(x):
    return tuple(int(d) for d in x.shape)


_KINDS = {}


def _kind(x):
    """'float32', 'int64', ... for a numpy array or a torch tensor."""
    k = _KINDS.get(x.dtype)
    if k is None:
        k = _KINDS[x.dtype] = str(x.dtype).split(".")[-1]
    return k


def _check_coords(x, name="xyz", dtypes=("float32", "float64")):
    """x must be [frames, atoms, 3] of one of `dtypes`."""
    if x.ndim != 3 or x.shape[2] != 3:
        raise ValueError(f"{name} must have shape (frames, atoms, 3), got {_shape(x)}")
    if _kind(x) not in dtypes:
        raise TypeError(f"{name} must be {' or '.join(dtypes)}, got {_kind(x)}")


def _check_buffer(x, name, dtype, count, exact=False):
    """x (or None) must hold `dtype` values, exactly / at least `count` of them.
    The library writes or reads that many through the raw pointer."""
    if x is None:
        return
    if _kind(x) != dtype:
        raise TypeError(f"{name} must be {dtype}, got {_kind(x)}")
    n = x.size if isinstance(x, np.ndarray) else x.numel()
    if (n != count) if exact else (n < count):
        need = f"{count}" if exact else f"at least {count}"
        raise ValueError(f"{name} must have {need} elements, got {n}")


def row_bands(n_frame, band_floats, row_align=1):
    """Band boundaries of a streamed triangle (gbr_row_bands): an int64 array
    cuts with cuts[0] = 0 and cuts[-1] = n_frame; raises ValueError when one
    row does not fit in a band."""
    cuts = np.zeros(int(n_frame) + 2, np.int64)
    nb = load().gbr_row_bands(int(n_frame), int(band_floats), int(row_align), cuts.ctypes.data, len(cuts))
    if nb < 0:
        raise ValueError(f"a band of {band_floats} floats cannot hold one row of {n_frame} frames")
    return cuts[: nb + 1].copy()


def output_count(n_ref, n_tgt, out_kind, row_begin=0, row_end=-1):
    return load().gbr_output_count(n_ref, n_tgt, out_kind, row_begin, row_end)


class Handle:
    """One gbr_handle (device memory, stream).  Not thread-safe."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = self.lib.gbr_create(device)
        if not self.h:
            raise GbrError(2, f"gbr_create({device}) failed (no usable CUDA device?)")
        self.device = device

    def close(self):
        if self.h:
            self.lib.gbr_destroy(self.h)
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
        if rc != GBR_OK:
            raise GbrError(rc, self.lib.gbr_last_error(self.h).decode())

    def set_option(self, key, value):
        self._check(self.lib.gbr_set_option(self.h, key, float(value)))

    def set_stream(self, stream_ptr):
        """Use a caller's cudaStream_t (an int pointer value, e.g.
        torch.cuda.current_stream().cuda_stream); None restores the handle's own."""
        self._check(self.lib.gbr_set_stream(self.h, stream_ptr))

    def selftest_bounded_wait(self, limit_cycles: int = 2_000_000):
        """Run the bounded-wait expiry self-test; returns (site code, cycles waited)."""
        site, waited = ctypes.c_int32(0), ctypes.c_int64(0)
        self._check(self.lib.gbr_selftest_bounded_wait(self.h, int(limit_cycles), ctypes.byref(site),
                                                       ctypes.byref(waited)))
        return site.value, waited.value

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.gbr_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def allpairs_raw(self, ref, tgt, n_ref, n_tgt, n_atom, dtype, ref_mass, tgt_mass, mode, out_kind,
                     precision, out, row_begin=0, row_end=-1):
        """Direct call with raw pointers / arrays (the C ABI, unchanged)."""
        rc = self.lib.gbr_allpairs(self.h, _ptr(ref), _ptr(tgt), dtype, n_ref, n_tgt, n_atom, _ptr(ref_mass),
                                   _ptr(tgt_mass), mode, out_kind, precision, _ptr(out), row_begin, row_end)
        self._check(rc)

    def allpairs(self, ref, tgt=None, ref_mass=None, tgt_mass=None, mode="fit", out_kind=None,
                 precision="fp32", out=None, row_begin=0, row_end=-1):
        """All-pairs RMSD (rms2d semantics).  ref/tgt: [frames, atoms, 3].

        Returns ``out`` (allocated like ``ref`` -- numpy or torch, same
        device -- when not given).  TRI for one set, FULL when ``tgt`` is given.
        """
        _check_coords(ref, "ref")
        n_ref, n_atom = int(ref.shape[0]), int(ref.shape[1])
        if tgt is not None:
            _check_coords(tgt, "tgt")
            if int(tgt.shape[1]) != n_atom or _kind(tgt) != _kind(ref):
                raise ValueError("tgt must have the atom count and dtype of ref")
        n_tgt = int(tgt.shape[0]) if tgt is not None else n_ref
        if out_kind is None:
            out_kind = TRI if tgt is None else FULL
        m = MODES[mode] if isinstance(mode, str) else mode
        p = PRECISIONS[precision] if isinstance(precision, str) else precision
        count = output_count(n_ref, n_tgt, out_kind, row_begin, row_end)
        if out is None:
            if isinstance(ref, np.ndarray):
                out = np.zeros(count, np.float32)
            else:
                import torch
                out = torch.zeros(count, dtype=torch.float32, device=ref.device)
        _check_buffer(out, "out", "float32", count)
        if tgt_mass is not None and isinstance(tgt_mass, np.ndarray):
            tgt_mass = np.ascontiguousarray(tgt_mass, dtype=np.float64)
        if ref_mass is not None and isinstance(ref_mass, np.ndarray):
            ref_mass = np.ascontiguousarray(ref_mass, dtype=np.float64)
        _check_buffer(tgt_mass, "tgt_mass", "float64", n_atom, exact=True)
        _check_buffer(ref_mass, "ref_mass", "float64", n_atom, exact=True)
        self.allpairs_raw(ref, tgt, n_ref, n_tgt, n_atom, _dtype_code(ref), ref_mass, tgt_mass, m, out_kind, p,
                          out, row_begin, row_end)
        return out

    def superpose(self, ref, xyz, mass=None, ref_mass=None, mode="fit", move=None):
        """Per-frame best fit onto one reference frame (the rms / align actions).

        ref: [atoms, 3]; xyz: [frames, atoms, 3] (numpy or torch, same dtype);
        move: optional [frames, n_move, 3] array of that dtype, moved in place.
        Returns (rmsd [F], rot [F, 3, 3], tgt_trans [F, 3], ref_trans [3]) as
        float64 arrays of the same kind and device as ``xyz``."""
        _check_coords(xyz)
        F, N = int(xyz.shape[0]), int(xyz.shape[1])
        if _shape(ref) != (N, 3) or _kind(ref) != _kind(xyz):
            raise ValueError(f"ref must have shape ({N}, 3) and the dtype of xyz")
        m = MODES[mode] if isinstance(mode, str) else mode
        if isinstance(xyz, np.ndarray):
            def mk(*shape):
                return np.zeros(shape, np.float64)
            if mass is not None:
                mass = np.ascontiguousarray(mass, dtype=np.float64)
            if ref_mass is not None:
                ref_mass = np.ascontiguousarray(ref_mass, dtype=np.float64)
        else:
            import torch

            def mk(*shape):
                return torch.zeros(shape, dtype=torch.float64, device=xyz.device)
        _check_buffer(mass, "mass", "float64", N, exact=True)
        _check_buffer(ref_mass, "ref_mass", "float64", N, exact=True)
        rmsd, rot, tt, rt = mk(F), mk(F, 3, 3), mk(F, 3), mk(3)
        n_move = 0 if move is None else int(move.shape[1])
        if move is not None:
            if _dtype_code(move) != _dtype_code(xyz):
                raise TypeError("move must have the dtype of xyz")
            if len(_shape(move)) != 3 or _shape(move)[0] != F or _shape(move)[2] != 3:
                raise ValueError(f"move must have shape ({F}, atoms, 3), got {_shape(move)}")
        self._check(self.lib.gbr_superpose(self.h, _ptr(ref), _ptr(xyz), _dtype_code(xyz), F, N, _ptr(ref_mass),
                                           _ptr(mass), m, _ptr(rmsd), _ptr(rot), _ptr(tt), _ptr(rt), _ptr(move),
                                           n_move))
        return rmsd, rot, tt, rt

    def cluster_centroids(self, xyz, members, offsets, mass=None, mode="fit"):
        """Cluster centroids (Metric_RMS::CalculateCentroid).

        xyz: [frames, atoms, 3] (numpy or torch); members (int32) and
        offsets (int64, [n_cluster + 1]): cluster c is members[offsets[c]:
        offsets[c + 1]] in visiting order.  Returns [n_cluster, atoms, 3]
        float64 of the same kind and device as ``xyz``."""
        _check_coords(xyz)
        F, N = int(xyz.shape[0]), int(xyz.shape[1])
        nc = int(offsets.shape[0]) - 1
        m = MODES[mode] if isinstance(mode, str) else mode
        if isinstance(xyz, np.ndarray):
            members = np.ascontiguousarray(members, dtype=np.int32)
            offsets = np.ascontiguousarray(offsets, dtype=np.int64)
            if mass is not None:
                mass = np.ascontiguousarray(mass, dtype=np.float64)
            out = np.zeros((max(nc, 0), N, 3), np.float64)
        else:
            import torch

            out = torch.zeros((max(nc, 0), N, 3), dtype=torch.float64, device=xyz.device)
        _check_buffer(members, "members", "int32", 0)
        _check_buffer(offsets, "offsets", "int64", max(nc + 1, 1), exact=True)
        _check_buffer(mass, "mass", "float64", N, exact=True)
        self._check(self.lib.gbr_cluster_centroids(self.h, _ptr(xyz), _dtype_code(xyz), F, N, _ptr(mass), m,
                                                   _ptr(members), _ptr(offsets), nc, _ptr(out)))
        return out

    def allpairs_batched(self, trajs, masses=None, mode="fit", precision="fp32"):
        """trajs: list of float32 [F_t, N_t, 3] arrays; returns list of TRI outputs."""
        n = len(trajs)
        for t, x in enumerate(trajs):
            _check_coords(x, f"trajs[{t}]", ("float32",))
        if masses is not None and len(masses) != n:
            raise ValueError("masses must have one entry per trajectory")
        outs = [np.zeros(max(int(t.shape[0]) * (int(t.shape[0]) - 1) // 2, 1), np.float32) for t in trajs]
        xyz = (ctypes.c_void_p * n)(*[_ptr(t) for t in trajs])
        nf = (ctypes.c_int64 * n)(*[int(t.shape[0]) for t in trajs])
        na = (ctypes.c_int32 * n)(*[int(t.shape[1]) for t in trajs])
        ms = None
        if masses is not None:
            masses = [None if m is None else np.ascontiguousarray(m, np.float64) for m in masses]
            for t, (mt, x) in enumerate(zip(masses, trajs)):
                _check_buffer(mt, f"masses[{t}]", "float64", int(x.shape[1]), exact=True)
            ms = (ctypes.c_void_p * n)(*[_ptr(m) for m in masses])
        op = (ctypes.c_void_p * n)(*[_ptr(o) for o in outs])
        m = MODES[mode] if isinstance(mode, str) else mode
        p = PRECISIONS[precision] if isinstance(precision, str) else precision
        rc = self.lib.gbr_allpairs_batched(self.h, n, ctypes.cast(xyz, ctypes.c_void_p),
                                           ctypes.cast(nf, ctypes.c_void_p), ctypes.cast(na, ctypes.c_void_p),
                                           None if ms is None else ctypes.cast(ms, ctypes.c_void_p), m, p,
                                           ctypes.cast(op, ctypes.c_void_p))
        self._check(rc)
        return [o[: int(t.shape[0]) * (int(t.shape[0]) - 1) // 2] for o, t in zip(outs, trajs)]

    def allpairs_stream(self, xyz, sink, mass=None, mode="fit", precision="tc", band_floats=0):
        """The triangle of one frame set in row bands (gbr_allpairs_stream).

        ``sink(row_begin, row_end, values)`` is called on this thread for each
        band in row order; ``values`` is a float32 view of the library's
        pinned staging, valid only during the call (copy what you keep).
        Returning False stops the call (GbrError code 7)."""
        _check_coords(xyz)
        n_frame, n_atom = int(xyz.shape[0]), int(xyz.shape[1])
        if mass is not None and isinstance(mass, np.ndarray):
            mass = np.ascontiguousarray(mass, dtype=np.float64)
        _check_buffer(mass, "mass", "float64", n_atom, exact=True)
        errors = []

        def _cb(user, rb, re, values, count):
            try:
                arr = np.ctypeslib.as_array(values, shape=(int(count),)) if count > 0 else np.zeros(0, np.float32)
                return 1 if sink(int(rb), int(re), arr) is False else 0
            except BaseException as e:  # noqa: BLE001 - re-raised after the call
                errors.append(e)
                return 1
        cb = BAND_SINK(_cb)
        m = MODES[mode] if isinstance(mode, str) else mode
        p = PRECISIONS[precision] if isinstance(precision, str) else precision
        rc = self.lib.gbr_allpairs_stream(self.h, _ptr(xyz), _dtype_code(xyz), n_frame, n_atom, _ptr(mass), m, p,
                                          int(band_floats), cb, None)
        if errors:
            raise errors[0]
        self._check(rc)

    def write_cmatrix(self, path, xyz, mass=None, mode="fit", precision="tc", frame_to_idx=None, sieve=1):
        """Pairwise cache of one frame set straight to a cpptraj binary
        cluster-matrix file (CTM version 2)."""
        _check_coords(xyz)
        n_frame, n_atom = int(xyz.shape[0]), int(xyz.shape[1])
        if mass is not None and isinstance(mass, np.ndarray):
            mass = np.ascontiguousarray(mass, dtype=np.float64)
        _check_buffer(mass, "mass", "float64", n_atom, exact=True)
        f2i = None
        n_orig = n_frame
        if frame_to_idx is not None:
            f2i = np.ascontiguousarray(frame_to_idx, dtype=np.int32)
            n_orig = len(f2i)
        m = MODES[mode] if isinstance(mode, str) else mode
        p = PRECISIONS[precision] if isinstance(precision, str) else precision
        rc = self.lib.gbr_write_cmatrix(self.h, os.fsencode(path), _ptr(xyz), _dtype_code(xyz), n_frame, n_atom,
                                        _ptr(mass), m, p, _ptr(f2i), n_orig, int(sieve))
        self._check(rc)

    def backward(self, xyz, mass=None, g=None, grad=None, rmsd_out=None):
        """dL/dxyz for L = sum_{i<j} g_ij RMSD_ij (float32 frames)."""
        _check_coords(xyz, dtypes=("float32",))
        n_frame, n_atom = int(xyz.shape[0]), int(xyz.shape[1])
        n_pairs = n_frame * (n_frame - 1) // 2
        if grad is None:
            if isinstance(xyz, np.ndarray):
                grad = np.zeros_like(xyz)
            else:
                import torch
                grad = torch.zeros_like(xyz)
        if mass is not None and isinstance(mass, np.ndarray):
            mass = np.ascontiguousarray(mass, dtype=np.float64)
        _check_buffer(mass, "mass", "float64", n_atom, exact=True)
        _check_buffer(g, "g", "float32", n_pairs)
        _check_buffer(grad, "grad", "float32", n_frame * n_atom * 3)
        _check_buffer(rmsd_out, "rmsd_out", "float32", n_pairs)
        rc = self.lib.gbr_rmsd_backward(self.h, _ptr(xyz), n_frame, n_atom, _ptr(mass), _ptr(g), _ptr(grad),
                                        _ptr(rmsd_out))
        self._check(rc)
        return grad


_default = {}


def default_handle(device: int = 0) -> Handle:
    h = _default.get(device)
    if h is None:
        h = _default[device] = Handle(device)
    return h


def allpairs_fp64_static(xyz, mass=None, mode="fit", out=None, stream=None):
    """gbr_allpairs_fp64_static: FP64 all-pairs RMSD with no allocation inside
    the library.  xyz ([F, N, 3] float32/float64), mass ([N] float64 or None)
    and out ([>= F(F-1)/2] float32, allocated here when None) must be CUDA
    tensors on one device; the call runs with that device current, on
    ``stream`` (a cudaStream_t value) or else on torch's current stream of
    that device.  Returns out."""
    import torch

    if not (isinstance(xyz, torch.Tensor) and xyz.is_cuda):
        raise ValueError("xyz must be a CUDA tensor")
    if xyz.dim() != 3 or xyz.shape[2] != 3:
        raise ValueError(f"xyz must have shape (frames, atoms, 3), got {tuple(xyz.shape)}")
    F, N = int(xyz.shape[0]), int(xyz.shape[1])
    dev = xyz.device
    n_out = max(F * (F - 1) // 2, 0)
    if mass is not None:
        if not (isinstance(mass, torch.Tensor) and mass.device == dev):
            raise ValueError("mass must be a CUDA tensor on the device of xyz")
        if mass.dtype != torch.float64 or mass.numel() != N:
            raise ValueError(f"mass must be float64 with {N} elements, got {mass.dtype} x {mass.numel()}")
    if out is None:
        out = torch.empty(n_out, dtype=torch.float32, device=dev)
    elif not (isinstance(out, torch.Tensor) and out.device == dev):
        raise ValueError("out must be a CUDA tensor on the device of xyz")
    elif out.dtype != torch.float32 or out.numel() < n_out:
        raise ValueError(f"out must be float32 with at least {n_out} elements, got {out.dtype} x {out.numel()}")
    m = MODES[mode] if isinstance(mode, str) else mode
    L = load()
    with torch.cuda.device(dev):
        st = torch.cuda.current_stream(dev).cuda_stream if stream is None else stream
        rc = L.gbr_allpairs_fp64_static(_ptr(xyz), _dtype_code(xyz), F, N, _ptr(mass), m, _ptr(out), st)
    if rc != GBR_OK:
        raise GbrError(rc, "gbr_allpairs_fp64_static failed")
    return out
