"""Builds and runs the drop-in test application (tests/dropin/nbs_app.c).

Two builds of the same application source:
* reference build (oracle/_ref/nbs_app_ref, made by oracle/build_ref.sh where
  the reference tree exists): the reference's PAMR/AMRD with amrd/mg.c;
* device build (tests/dropin/_build/nbs_app_dev, made here): the oracle
  port's PAMR environment (oracle/port/pamr_env.c) with libamrd_mg_gb300 in
  place of amrd/mg.c, -DDEVICE_MG.

TEST INFRASTRUCTURE: used by tests/ and tests/golden/make_golden.py.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build")
DEV_APP = os.path.join(OUT, "nbs_app_dev")
REF_APP = os.path.join(ROOT, "oracle", "_ref", "nbs_app_ref")
LINK_CHECK_APP = os.path.join(ROOT, "oracle", "_ref", "nbs_app_dropin_linked")


def cuda_lib() -> str:
    from pamr_amrd_gb300 import build as B
    return os.path.join(B.cuda_home(), "lib64")


def build_device_app(force: bool = False) -> str:
    """the application over the port's PAMR environment, linked with
    libamrd_mg_gb300.so (which the app's executable resolves PAMR/AMRD for,
    hence --export-dynamic)"""
    from pamr_amrd_gb300 import build as B
    B.build()
    srcs = [os.path.join(HERE, "nbs_app.c"), os.path.join(ROOT, "oracle", "port", "pamr_env.c"),
            os.path.join(ROOT, "oracle", "mg_ops.c"), os.path.join(ROOT, "oracle", "m_util_r8.c"),
            os.path.join(ROOT, "oracle", "bo_ops.c")]
    deps = srcs + [B.LIB_AMRD_MG, os.path.join(ROOT, "oracle", "port", "mg_port.c"),
                   os.path.join(HERE, "dropin_case.h")]
    os.makedirs(OUT, exist_ok=True)
    if force or not os.path.exists(DEV_APP) or os.path.getmtime(DEV_APP) < max(os.path.getmtime(d) for d in deps):
        pkg = os.path.dirname(B.LIB)
        cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-DDEVICE_MG",
               "-I" + os.path.join(ROOT, "oracle"), "-I" + B.CSRC, "-I" + os.path.join(ROOT, "include"),
               "-I" + HERE] + srcs + [
            "-o", DEV_APP, "-L" + pkg, "-lamrd_mg_gb300", "-lpamr_gb300", "-L" + cuda_lib(), "-lcudart", "-lm",
            "-Wl,--export-dynamic", "-Wl,-rpath," + pkg, "-Wl,-rpath," + cuda_lib()]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("building the device app failed:\n" + r.stdout + r.stderr)
    return DEV_APP


def write_case(case, path: str, mode: int = 0, arg: int = 0, level: int = 1):
    p = case.params
    if case.nsrc != 2:
        raise ValueError("the drop-in application reads two sources")
    out = [struct.pack("<8i", case.dim, len(case.grids), mode, arg, level, int(case.nvar == 2), 0, 0)]
    out.append(struct.pack("<6d", *(list(case.base_bbox) + [0.0] * (6 - len(case.base_bbox)))))
    out.append(struct.pack("<4i", *case.base_shape, 0))
    out.append(struct.pack("<10i", p.pre_swp, p.pst_swp, p.max_iter, p.min_iter, p.max_citer, p.min_cwidth,
                           p.restr_u, p.restr_res, p.restr_src, case.restr_src_k(1)))
    out.append(struct.pack("<4d", p.tol, p.crtol, p.w0_r, p.w0_i))
    for i, g in enumerate(case.grids):
        out.append(struct.pack("<4i6d", g.level, *g.shape, *(list(g.bbox) + [0.0] * (6 - len(g.bbox)))))
        for a in [case.u0[i]] + [case.var(v)[i] for v in range(1, case.nvar)] + [case.src[i], case.source(1)[i]]:
            out.append(np.ascontiguousarray(a, dtype="<f8").tobytes())
    with open(path, "wb") as f:
        f.write(b"".join(out))


def parse(buf: bytes, nvar: int = 1) -> dict:
    iters, nres = struct.unpack_from("<2i", buf, 0)
    off = 8
    res = np.frombuffer(buf, dtype="<f8", count=nres, offset=off).copy()
    off += 8 * nres
    (nh,) = struct.unpack_from("<i", buf, off)
    off += 4
    rec = np.frombuffer(buf, dtype=np.dtype([("kind", "<i4"), ("L", "<i4"), ("norm", "<f8")]), count=nh,
                        offset=off).copy()
    off += 16 * nh
    grids = []
    while off < len(buf):
        lev, s0, s1, s2 = struct.unpack_from("<4i", buf, off)
        off += 16
        bb = struct.unpack_from("<6d", buf, off)
        off += 48
        n = s0 * s1 * s2
        u = np.frombuffer(buf, dtype="<f8", count=n, offset=off).copy()
        off += 8 * n
        cm = np.frombuffer(buf, dtype="<f8", count=n, offset=off).copy()
        off += 8 * n
        grid = {"level": lev, "shape": (s0, s1, s2), "bbox": bb, "u": u, "cmask": cm}
        if nvar == 2:   # the second elliptic variable of a coupled case
            grid["w"] = np.frombuffer(buf, dtype="<f8", count=n, offset=off).copy()
            off += 8 * n
        grids.append(grid)
    return {"iters": iters, "res": res, "hooks": rec, "grids": grids}


def run(binary: str, case, mode: int = 0, arg: int = 0, level: int = 1, env=None, timeout: float = 1200) -> dict:
    from oracle import refrun
    with tempfile.TemporaryDirectory() as td:
        cf, pf, of = (os.path.join(td, n) for n in ("case.bin", "case.param", "out.bin"))
        write_case(case, cf, mode, arg, level)
        with open(pf, "w") as f:
            f.write(refrun.param_file(case))
        e = dict(os.environ)
        e.update(env or {})
        r = subprocess.run([binary, cf, pf, of], capture_output=True, text=True, timeout=timeout, cwd=td, env=e)
        if r.returncode != 0:
            raise RuntimeError(f"{os.path.basename(binary)} failed ({r.returncode}): {r.stdout[-3000:]} {r.stderr[-3000:]}")
        with open(of, "rb") as f:
            out = parse(f.read(), case.nvar)
    out["stdout"] = r.stdout
    return out


def finest_residuals(out: dict) -> np.ndarray:
    """per-cycle finest residual of a reference-build solve, from its hook
    log (the residual hook's max over the finest level's grids at the end of
    each cycle, amrd/mg.c:194)"""
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    import golden_cases as G
    h = out["hooks"]
    lf = max(g["level"] for g in out["grids"])
    hooks = {"kind": h["kind"], "L": h["L"], "norm": h["norm"]}
    # hook levels are MG levels: the finest MG level is the largest seen
    lf = int(h["L"].max()) if len(h) else lf
    return G.finest_residuals(hooks, lf)
