"""Run the reference's own multigrid solve (oracle/_ref/ref_mg) on a Case.

TEST INFRASTRUCTURE (oracle only): imported by tests/ and by the golden
fixture script. ``oracle/_ref/ref_mg`` is compiled from the reference's C
sources by ``oracle/build_ref.sh`` where the reference tree exists; on other
machines this module reports that it is unavailable.

The parameter file written here is an AMRD run-time file that the
reference's ``init_context`` (amrd/io.c:36) reads: one elliptic variable
``u`` (mg_sync, mg_interp2, HW restriction) whose residual ``u_res`` uses
full weighting, and one source ``rho`` defined as a hyperbolic variable so
it lives in both hierarchies and is restricted onto pure MG levels
(examples/nbs/nbs.fparam pattern). Operators with several sources (the nbs
potential reads phi_r and phi_i) get ``rho1``, ``rho2`` .. beside ``rho``.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "ref_mg")

_OP_NAME = {1: "STRAIGHT", 2: "HW", 3: "FW"}
# the gfns ref_main.c reports, in its order (src1.. only for operators with several sources)
GFN_KEYS = ("u", "res", "lop", "rhs", "cmask", "src", "src1", "src2", "src3")
# source variables as oracle/ref_main.c names them
SRC_NAMES = ("rho", "rho1", "rho2", "rho3")
# elliptic variables as oracle/ref_main.c names them
VAR_NAMES = ("u", "w")


def available() -> bool:
    return os.path.exists(REF_BIN)


def param_file(case, amr_interp_order: int = 0, transfer_order: int = 0) -> str:
    """AMRD run-time parameters of ``case``; amr_interp_order 2 or 4 also
    lists u in amr_interp2/amr_interp4 (its AMR interpolation order,
    amrd/io.c:771-772); transfer_order 2 or 4 lists u and the sources in
    amr_transfer2/amr_transfer4 (their regrid_transfer order,
    amrd/io.c:778-779)"""
    p = case.params
    dim = case.dim
    lines = [
        "echo_params := 0",
        "pamr_trace_lev := 0",
        "MG_trace := 0",
        "MG_DV_trace := 0",
        f"dim := {dim}",
        "base_shape := [" + " ".join(str(case.base_shape[d]) for d in range(dim)) + "]",
        "base_bbox := [" + " ".join(repr(float(b)) for b in case.base_bbox[:2 * dim]) + "]",
        f"max_lev := {case.num_levels}",
        "num_evo_tl := 2",
        "rho_sp := 2",
        "rho_tm := 2",
        f'num_hyperbolic_vars := {case.nsrc}',
        'hyperbolic_vars := [ ' + " ".join(f'"{n}"' for n in SRC_NAMES[:case.nsrc]) + ' ]',
        f'num_elliptic_vars := {case.nvar}',
        'elliptic_vars := [ ' + " ".join(f'"{n}"' for n in VAR_NAMES[:case.nvar]) + ' ]',
        f"num_mg_sync := {case.nvar}",
        'mg_sync := [ ' + " ".join(f'"{n}"' for n in VAR_NAMES[:case.nvar]) + ' ]',
        f"num_mg_interp2 := {case.nvar}",
        'mg_interp2 := [ ' + " ".join(f'"{n}"' for n in VAR_NAMES[:case.nvar]) + ' ]',
        f"MG_pre_swp := {p.pre_swp}",
        f"MG_pst_swp := {p.pst_swp}",
        f"MG_max_iter := {p.max_iter}",
        f"MG_min_iter := {p.min_iter}",
        f"MG_max_citer := {p.max_citer}",
        f"MG_tol := {p.tol!r}",
        f"MG_crtol := {p.crtol!r}",
        f"MG_w0_r := {p.w0_r!r}",
        f"MG_w0_i := {p.w0_i!r}",
        "min_mg_cwidth := [" + " ".join(str(p.min_cwidth) for _ in range(dim)) + "]",
    ]
    hw, fw = [], []
    srcs = [(SRC_NAMES[k], case.restr_src_k(k)) for k in range(case.nsrc)]
    ell = [(n, p.restr_u) for n in VAR_NAMES[:case.nvar]] + [(n + "_res", p.restr_res) for n in VAR_NAMES[:case.nvar]]
    for name, op in ell + srcs:
        if op == 2:
            hw.append(name)
        elif op == 3:
            fw.append(name)
        elif op != 0:
            raise ValueError("the AMRD parameter interface offers HW or FW restriction only")
    # f_res defaults to HW (amrd/io.c:865); it is listed only to select FW
    hw = [n for n in hw if not n.endswith("_res")]
    if hw:
        lines += [f"num_mg_hw_restr := {len(hw)}",
                  "mg_hw_restr := [ " + " ".join(f'"{n}"' for n in hw) + " ]"]
    if fw:
        lines += [f"num_mg_fw_restr := {len(fw)}",
                  "mg_fw_restr := [ " + " ".join(f'"{n}"' for n in fw) + " ]"]
    if p.interp_order != 2:
        raise ValueError("AMRD's coarse-grid correction interpolates with mg_interp2 only")
    if amr_interp_order:
        lines += [f"num_amr_interp{amr_interp_order} := 1", f'amr_interp{amr_interp_order} := [ "u" ]']
    if transfer_order:
        names = ["u"] + list(SRC_NAMES[:case.nsrc])
        lines += [f"num_amr_transfer{transfer_order} := {len(names)}",
                  f"amr_transfer{transfer_order} := [ " + " ".join(f'"{n}"' for n in names) + " ]"]
    return "\n".join(lines) + "\n"


def case_bytes(case) -> bytes:
    """header (dim, pde, grids, coarsest AMR level of the MG hierarchy),
    then per grid level, shape, bbox, u and each source"""
    out = [struct.pack("<4i", case.dim, case.pde, len(case.grids), case.min_level)]
    for i, (g, u) in enumerate(zip(case.grids, case.u0)):
        bb = list(g.bbox) + [0.0] * (6 - len(g.bbox))
        out.append(struct.pack("<4i6d", g.level, *g.shape, *bb))
        out.append(np.ascontiguousarray(u, dtype="<f8").tobytes())
        for v in range(1, case.nvar):
            out.append(np.ascontiguousarray(case.var(v)[i], dtype="<f8").tobytes())
        for k in range(case.nsrc):
            out.append(np.ascontiguousarray(case.source(k)[i], dtype="<f8").tobytes())
    return b"".join(out)


def _records(buf: bytes):
    off = 0
    while off < len(buf):
        tag, n = struct.unpack_from("<iq", buf, off)
        off += 12
        yield tag, buf[off:off + n]
        off += n


def run_reference(case, log_ops: bool = False, workdir: str | None = None,
                  timeout: float = 3600, amr_interp=None, regrid=None) -> dict:
    """Runs ref_mg on ``case``; returns iterations, hook log, MG hierarchy,
    cmask arrays, final u per input grid and (optionally) the m_util_r8 op log.
    With amr_interp = (lc, width, order) the solve is replaced by one
    PAMR_interp (width 0) or PAMR_AMR_bdy_interp (width > 0) of u from AMR
    level lc to lc+1 with interpolation order 2 or 4; "u" then holds the
    AMR grids after it. With regrid = (new_case, min_lev, order) the solve is
    replaced by a second PAMR_compose_hierarchy over levels min_lev.. of
    new_case's grids, u and the sources transferred with that
    regrid_transfer order; "regrid" then lists every AMR grid after it
    (level, shape, bbox, u, sources) in PAMR's order."""
    if not available():
        raise RuntimeError("oracle/_ref/ref_mg is not built (oracle/build_ref.sh)")
    with tempfile.TemporaryDirectory(dir=workdir) as td:
        pf = os.path.join(td, "case.param")
        cf = os.path.join(td, "case.bin")
        of = os.path.join(td, "out.bin")
        with open(pf, "w") as f:
            f.write(param_file(case, amr_interp[2] if amr_interp else 0, regrid[2] if regrid else 0))
        with open(cf, "wb") as f:
            f.write(case_bytes(case))
        extra = ["1" if log_ops else "0"] + ([f"interp:{amr_interp[0]}:{amr_interp[1]}"] if amr_interp else [])
        if regrid:
            nf = os.path.join(td, "new.bin")
            with open(nf, "wb") as f:
                f.write(case_bytes(regrid[0]))
            extra = ["1" if log_ops else "0", f"regrid:{regrid[1]}:{nf}"]
        r = subprocess.run([REF_BIN, pf, cf, of] + extra,
                           capture_output=True, text=True, timeout=timeout, cwd=td)
        if r.returncode != 0:
            raise RuntimeError(f"ref_mg failed ({r.returncode}): {r.stdout[-2000:]} {r.stderr[-2000:]}")
        with open(of, "rb") as f:
            buf = f.read()
    res = {"iters": 0, "hooks": None, "mgh": [], "masks": [], "u": [], "ops": [],
           "regrid": [], "u_extra": [], "stdout": r.stdout}
    pending_mask = None
    for tag, p in _records(buf):
        if tag == 1:
            res["iters"] = struct.unpack("<i", p)[0]
        elif tag == 2:
            v = struct.unpack(f"<{len(p) // 4}i", p)
            res["gfn"] = {k: g for k, g in zip(GFN_KEYS, v) if g > 0}
        elif tag == 3:
            a = np.frombuffer(p, dtype=np.dtype([("kind", "<i4"), ("L", "<i4"), ("idx", "<i4"),
                                                 ("pad", "<i4"), ("norm", "<f8")]))
            res["hooks"] = a.copy()
        elif tag == 4:
            L, idx, s0, s1, s2, co = struct.unpack_from("<6i", p)
            bb = struct.unpack_from("<6d", p, 24)
            res["mgh"].append({"L": L, "idx": idx, "shape": (s0, s1, s2), "coarsest": co,
                               "bbox": bb})
        elif tag == 5:
            pending_mask = struct.unpack("<4i", p)
        elif tag == 6:
            kind, L, idx, n = pending_mask
            res["masks"].append({"kind": ("bdy", "child")[kind], "L": L, "idx": idx,
                                 "mask": np.frombuffer(p, dtype="<f8").copy()})
        elif tag == 7:
            res["u"].append(np.frombuffer(p, dtype="<f8").copy())
        elif tag == 8:
            v = np.frombuffer(p, dtype="<i4").copy()
            res["ops"].append(v)
        elif tag == 12:   # the other elliptic variables, grid by grid
            res["u_extra"].append(np.frombuffer(p, dtype="<f8").copy())
        elif tag == 9:
            L, s0, s1, s2 = struct.unpack_from("<4i", p)
            res["regrid"].append({"L": L, "shape": (s0, s1, s2), "bbox": struct.unpack_from("<6d", p, 16),
                                  "u": None, "src": []})
        elif tag == 10:
            res["regrid"][-1]["u"] = np.frombuffer(p, dtype="<f8").copy()
        elif tag == 11:
            res["regrid"][-1]["src"].append(np.frombuffer(p, dtype="<f8").copy())
    if res["ops"]:
        res["ops"] = np.stack(res["ops"])
    return res


def finest_residuals(ref: dict, lf: int) -> np.ndarray:
    """per-V-cycle finest-level residual: the last residual-hook value on
    level lf in each cycle (amrd/mg.c:194), max over that level's grids."""
    h = ref["hooks"]
    out = []
    cur = []
    for rec in h:
        if rec["kind"] == 1 and rec["L"] == lf:
            cur.append(rec)
    # residual hooks on lf come in groups: [down (if lf>1)] then [final];
    # group consecutive calls by position in the log
    groups = []
    last_pos = None
    pos = np.nonzero((h["kind"] == 1) & (h["L"] == lf))[0]
    for p in pos:
        if last_pos is not None and p == last_pos + 1:
            groups[-1].append(p)
        else:
            groups.append([p])
        last_pos = p
    for g in groups:
        out.append(max(float(h["norm"][i]) for i in g))
    out = np.array(out)
    return out[1::2] if lf > 1 else out
