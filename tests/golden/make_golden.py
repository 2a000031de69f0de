"""Generate the committed golden fixtures for the all-pairs RMSD path.

Run in a container where the reference tree is mounted (default
/root/reference); the outputs are small .npz files that travel with the repo.

1. tz2_rms2d.npz -- inputs and expected outputs of test/Test_2DRMS/RunTest.sh
   (reference units 1, 2, 5, 6 and 8), re-derived from test/tz2.parm7 and
   test/tz2.crd (the ASCII copy of the tz2.nc trajectory the test reads):
     unit 1/8  `2drms crd1 :3-7`          -> rmsd.dat.save   (fit; qrmsd too)
     unit 2    `2drms crd1 :3-7 mass`     -> rmsd.mass.dat.save
     unit 5    `2drms :2 :11`             -> trp.dat.save    (tgt :2, ref :11, FULL)
     unit 6    `rms first :2-12@CA` then `2drms crd1 :2 nofit` -> nofit.dat.save
     unit 4    `2drms crd1 :3-7 rmsout dme.dat dme` -> dme.dat.save (same frames as unit 1)
   Coordinates are stored as float32 because the implicit COORDS set of those
   runs holds single precision (src/CompactFrameArray.h:75-76).
2. ref_pairs.npz -- FP64 RMSDs produced by cpptraj's own Frame code (built by
   `make -C oracle ref`) on seeded synthetic frames, for fit/nofit/qrmsd with
   and without mass weighting, and for dme (Frame::DISTRMSD).  This pins the restatement where the reference
   tree is absent.
3. tz2_cluster_cmatrix.npz -- the pairwise cache of test/Test_Cluster's first
   unit (`cluster C1 :2-10 ... nofit savepairdist ... pairdist Cmatrix.cmatrix`
   on all 101 tz2 frames): distances from cpptraj's own Metric_RMS arithmetic
   (frame f1 as target, RMSD_NoFit against f2) and the file bytes from its own
   Cmatrix_Binary::WriteCmatrix, for the full cache and for a regular sieve of
   3 (frames 0, 3, 6, ... kept).
4. ref_superpose.npz -- the per-frame fit of the rms / align actions run by
   cpptraj's own code (RMSD_CenteredRef with rotation and translation, then
   Trans_Rot_Trans of a larger "move" atom set), mass-weighted and not, on
   seeded synthetic frames.
5. ref_centroids.npz -- cluster centroids built by cpptraj's own Frame code in
   the steps of Metric_RMS::CalculateCentroid (fit: RMSD_CenteredRef onto the
   running sum, Rotate, +=, Divide; nofit: the plain sum), mass-weighted and
   not, for seeded synthetic frames split into 5 clusters (one of them empty)
   by seeded labels.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("CPPTRAJ_REFERENCE", "/root/reference")


def read_parm7(path):
    """Minimal Amber parm7 reader: atom names, masses, residue pointers."""
    flags = {}
    cur = None
    fmt = None
    with open(path) as fh:
        for line in fh:
            if line.startswith("%FLAG"):
                cur = line.split()[1]
                flags[cur] = []
            elif line.startswith("%FORMAT"):
                fmt = line[line.index("(") + 1: line.index(")")]
                flags[cur + "__fmt"] = fmt
            elif cur is not None and not line.startswith("%"):
                flags[cur].append(line.rstrip("\n"))

    def fixed(name, width, conv):
        out = []
        for ln in flags[name]:
            for k in range(0, len(ln), width):
                field = ln[k:k + width]
                if field.strip():
                    out.append(conv(field))
        return out

    natom = fixed("POINTERS", 8, int)[0]
    names = [s.strip() for s in fixed("ATOM_NAME", 4, str)][:natom]
    mass = np.array(fixed("MASS", 16, float)[:natom])
    respt = np.array(fixed("RESIDUE_POINTER", 8, int))
    return natom, names, mass, respt


def residue_of_atom(natom, respt):
    res = np.zeros(natom, dtype=np.int64)
    for r, start in enumerate(respt):
        res[start - 1:] = r + 1  # 1-based residue numbers
    return res


def read_crd(path, natom):
    with open(path) as fh:
        fh.readline()  # title
        vals = []
        for line in fh:
            for k in range(0, len(line.rstrip("\n")), 8):
                f = line[k:k + 8]
                if f.strip():
                    vals.append(float(f))
    v = np.array(vals)
    nf = len(v) // (3 * natom)
    return v[: nf * 3 * natom].reshape(nf, natom, 3)


def residue_mask(res, lo, hi):
    return np.nonzero((res >= lo) & (res <= hi))[0]


def kabsch_fit_all(frames, sel):
    """`rms first <sel>`: fit each frame onto frame 0 using atoms `sel`
    (geometric centres, proper rotation) and move all atoms."""
    ref = frames[0][sel]
    rc = ref.mean(axis=0)
    out = np.empty_like(frames)
    for f in range(len(frames)):
        x = frames[f][sel]
        xc = x.mean(axis=0)
        H = (x - xc).T @ (ref - rc)
        U, _, Vt = np.linalg.svd(H)
        d = np.sign(np.linalg.det(Vt.T @ U.T))
        R = Vt.T @ np.diag([1.0, 1.0, d]) @ U.T
        out[f] = (frames[f] - xc) @ R.T + rc
    return out


def read_square2d(path):
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#"):
                continue
            parts = line.split()
            if parts:
                rows.append([float(p) for p in parts[1:]])
    return np.array(rows)


def make_tz2():
    test = os.path.join(REF, "test")
    natom, names, mass, respt = read_parm7(os.path.join(test, "tz2.parm7"))
    res = residue_of_atom(natom, respt)
    frames = read_crd(os.path.join(test, "tz2.crd"), natom)[:10]
    m37 = residue_mask(res, 3, 7)
    m2 = residue_mask(res, 2, 2)
    m11 = residue_mask(res, 11, 11)
    ca = np.array([a for a in residue_mask(res, 2, 12) if names[a] == "CA"])
    fitted = kabsch_fit_all(frames, ca).astype(np.float32)
    f32 = frames.astype(np.float32)
    d = os.path.join(test, "Test_2DRMS")
    np.savez_compressed(
        os.path.join(HERE, "tz2_rms2d.npz"),
        fit_xyz=np.ascontiguousarray(f32[:, m37]),
        fit_mass=mass[m37],
        trp_tgt_xyz=np.ascontiguousarray(f32[:, m2]),
        trp_ref_xyz=np.ascontiguousarray(f32[:, m11]),
        trp_tgt_mass=mass[m2],
        trp_ref_mass=mass[m11],
        nofit_xyz=np.ascontiguousarray(fitted[:, m2]),
        nofit_mass=mass[m2],
        rmsd_save=read_square2d(os.path.join(d, "rmsd.dat.save")),
        rmsd_mass_save=read_square2d(os.path.join(d, "rmsd.mass.dat.save")),
        trp_save=read_square2d(os.path.join(d, "trp.dat.save")),
        nofit_save=read_square2d(os.path.join(d, "nofit.dat.save")),
        dme_save=read_square2d(os.path.join(d, "dme.dat.save")),
    )
    print("tz2_rms2d.npz: atoms", len(m37), len(m2), len(m11), "CA", len(ca))


def make_ref_pairs():
    sys.path.insert(0, ROOT)
    import oracle
    from cpptraj_gb300 import synth

    oracle.build(with_ref=True)
    X, m = synth.trajectory(11, 24, 157, 0.05, 3.0, np.float32, True)
    rng = np.random.default_rng(5)
    pi = rng.integers(0, 24, 200)
    pj = rng.integers(0, 24, 200)
    keep = pi != pj
    pi, pj = pi[keep], pj[keep]
    res = {"xyz": X, "mass": m, "pi": pi, "pj": pj}
    for mode, tag in ((oracle.FIT, "fit"), (oracle.NOFIT, "nofit")):
        for wt, mm in (("w", m), ("u", None)):
            res[f"{tag}_{wt}"] = oracle.pairs_f64(X, pi, pj, mass=mm, mode=mode, use_reference_code=True)
    # rms2d TRI float32 output of the reference for fit / qrmsd / nofit, weighted.
    for mode, tag in ((oracle.FIT, "fit"), (oracle.QCP, "qcp"), (oracle.NOFIT, "nofit"), (oracle.DME, "dme")):
        res[f"tri_{tag}"] = oracle.allpairs(X, tgt_mass=m, mode=mode, use_reference_code=True)
    res["dme_u"] = oracle.pairs_f64(X, pi, pj, mode=oracle.DME, use_reference_code=True)
    np.savez_compressed(os.path.join(HERE, "ref_pairs.npz"), **res)
    print("ref_pairs.npz:", len(pi), "pairs")


def make_cluster_cmatrix():
    sys.path.insert(0, ROOT)
    import tempfile

    import oracle

    oracle.build(with_ref=True)
    test = os.path.join(REF, "test")
    natom, names, mass, respt = read_parm7(os.path.join(test, "tz2.parm7"))
    res = residue_of_atom(natom, respt)
    frames = read_crd(os.path.join(test, "tz2.crd"), natom)
    sel = residue_mask(res, 2, 10)
    X = np.ascontiguousarray(frames[:, sel].astype(np.float32))
    out = {"xyz": X}

    def cache(kept):
        n = len(kept)
        f1, f2 = np.triu_indices(n, 1)
        # Metric_RMS::FrameDist(f1, f2): frm1 (f1) is the target, RMSD_NoFit against frm2
        d = oracle.pairs_f64(X, kept[f2], kept[f1], mode=oracle.NOFIT, use_reference_code=True)
        return d.astype(np.float32)

    for tag, step in (("full", 1), ("sieve3", 3)):
        F = X.shape[0]
        kept = np.arange(0, F, step)
        f2i = np.full(F, -1, np.int32)
        f2i[kept] = np.arange(len(kept), dtype=np.int32)
        tri = cache(kept)
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "c.cmatrix")
            oracle.ref_write_cmatrix(path, tri, f2i, step)
            out[f"ctm_{tag}"] = np.frombuffer(open(path, "rb").read(), dtype=np.uint8)
        out[f"f2i_{tag}"] = f2i
        out[f"tri_{tag}"] = tri
    np.savez_compressed(os.path.join(HERE, "tz2_cluster_cmatrix.npz"), **out)
    print("tz2_cluster_cmatrix.npz:", X.shape, {k: v.shape for k, v in out.items() if k.startswith("ctm")})


def make_ref_superpose():
    sys.path.insert(0, ROOT)
    import oracle
    from cpptraj_gb300 import synth

    oracle.build(with_ref=True)
    X, m = synth.trajectory(21, 30, 157, 0.05, 3.0, np.float32, True)
    move, _ = synth.trajectory(22, 30, 301, 0.5, 1.0, np.float64, False)
    res = {"xyz": X, "mass": m, "move": move}
    for tag, mm in (("w", m), ("u", None)):
        r, rot, tt, rt, mv = oracle.superpose_f64(X[5], X, mass=mm, move=move, use_reference_code=True)
        res.update({f"rmsd_{tag}": r, f"rot_{tag}": rot, f"tgt_trans_{tag}": tt, f"ref_trans_{tag}": rt,
                    f"moved_{tag}": mv})
    np.savez_compressed(os.path.join(HERE, "ref_superpose.npz"), **res)
    print("ref_superpose.npz:", X.shape, move.shape)


def make_ref_centroids():
    sys.path.insert(0, ROOT)
    import oracle
    from cpptraj_gb300 import synth

    oracle.build(with_ref=True)
    X, m = synth.trajectory(31, 90, 67, 0.3, 2.5, np.float32, True)
    labels = np.random.default_rng(32).integers(-1, 4, 90)  # -1: noise; cluster 4 stays empty
    members, offsets = oracle.members_offsets(labels, 5)
    res = {"xyz": X, "mass": m, "members": members, "offsets": offsets}
    for tag, mm, mode in (("fit_w", m, oracle.FIT), ("fit_u", None, oracle.FIT), ("nofit", None, oracle.NOFIT)):
        res[tag] = oracle.cluster_centroids_f64(X, members, offsets, mass=mm, mode=mode, use_reference_code=True)
    np.savez_compressed(os.path.join(HERE, "ref_centroids.npz"), **res)
    print("ref_centroids.npz:", X.shape, offsets)


if __name__ == "__main__":
    make_tz2()
    make_ref_pairs()
    make_cluster_cmatrix()
    make_ref_superpose()
    make_ref_centroids()
