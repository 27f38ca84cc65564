"""Drive the reference solver's own C code (built single-rank into oracle/_ref/) on
synthetic unit-cube forests, and read back its leaf dumps.

Test infrastructure: only tests/, tests/golden/make_golden.py and the CPU-baseline leg
of bench.py use this module.  It writes the reference's input files

  <case>.nd / .el        nodes and hex trees (format read by createtopo.c:26-65)
  <case>.ba .. .bd       boundary faces per bc code 1..4 (format read by boundary.c:32-36)
  <case>.ct              control file (positional lines read by inputset.c:31-125)
  <case>.m0ct            model-0 material tail (m0_input.c:14-33, see harness.c)
  <case>.ic / <case>.rf  initial state and refinement target read by harness.c

runs `forestfv_ref <case> <run>` and parses `<run>.init.bin` / `<run>.final.bin`.

Hex node order.  The reference derives face normals from node order
(normalvector.c:23-29 with the face-node table operatetp.c:60-69) and volumes from a
signed six-tet split (meshproperties.c:76-124).  Its update S = SN - DT/Vol * RHS with
RHS = sum of -A (F.n + HLLC correction) (RK.c:25, m0_residual.c:179-183) is a
conservative upwind scheme only when those normals point INTO the cell and the volume
comes out negative, i.e. for the node layout in which node k of a tree sits at
(x, y, z) = (bit1(k), bit0(k), bit2(k)).  `LAYOUT_INWARD` is that layout; the other
(`LAYOUT_OUTWARD`, node k at (bit0, bit1, bit2)) makes the reference anti-diffusive and
is only used by a test that shows so.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(HERE, "_ref", "forestfv_ref")
# the reference's C sources, read where they lie (FFV_REFERENCE_SRC, or the checkout's place
# in this build container); absent on machines without the reference
REF_SRC = os.environ.get("FFV_REFERENCE_SRC", "/root/reference/src/c")

# corner k of a hex tree/child -> (x, y, z) bit positions
LAYOUT_INWARD = ((1, 0, 2),)   # x = bit1, y = bit0, z = bit2
LAYOUT_OUTWARD = ((0, 1, 2),)  # x = bit0, y = bit1, z = bit2

# hex face -> its four nodes, operatetp.c:64-69 (fcnd2elnd, typ 0)
FACE_NODES = ((0, 1, 5, 4), (3, 7, 5, 1), (2, 6, 7, 3), (2, 0, 4, 6), (2, 3, 1, 0), (6, 4, 5, 7))


def corner_xyz(k: int, layout) -> tuple[int, int, int]:
    bx, by, bz = layout[0]
    return ((k >> bx) & 1, (k >> by) & 1, (k >> bz) & 1)


def morton_key(ix: int, iy: int, iz: int, nbits: int, layout) -> int:
    """Interleave so that the child index (corner bits in `layout`) is the fastest digit."""
    bx, by, bz = layout[0]
    key = 0
    for b in range(nbits):
        key |= ((ix >> b) & 1) << (3 * b + bx)
        key |= ((iy >> b) & 1) << (3 * b + by)
        key |= ((iz >> b) & 1) << (3 * b + bz)
    return key


def ref_available() -> bool:
    return os.path.isfile(REF_BIN) and os.access(REF_BIN, os.X_OK)


def build_ref(quiet: bool = True) -> bool:
    """Compile the reference into oracle/_ref with oracle/ref/Makefile (needs its sources)."""
    if not os.path.isdir(REF_SRC):
        return ref_available()
    cmd = ["make", "-C", os.path.join(HERE, "ref"), f"-j{os.cpu_count() or 4}", f"REF={REF_SRC}"]
    r = subprocess.run(cmd, capture_output=quiet, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + (r.stdout or "") + (r.stderr or ""))
    return ref_available()


@dataclass
class Case:
    """A unit-cube forest of tx*ty*tz cubic hex trees refined to `level` (trees are
    level 1 in the reference, so level=l gives 2**(l-1) cells per tree edge)."""
    trees: tuple[int, int, int] = (4, 4, 4)
    level: int = 2
    model: int = 0
    steps: int = 1
    dt: float = 1e-3
    rk_steps: int = 2
    order: int = 2
    gamma: float = 1.4
    pinf: float = 0.0
    ic: str = "split 0 0.5 1 0 0 0 1 0.125 0 0 0 0.1"
    refine: str | None = None          # harness .rf line, e.g. "sphere .5 .5 .5 .25 3 2"
    bc: tuple[int, ...] = (2, 2, 2, 2, 2, 2)   # per side -x,+x,-y,+y,-z,+z
    layout: tuple = LAYOUT_INWARD
    extra: dict = field(default_factory=dict)
    # model 5: dict with avf_lim, prelax, amin and per-material lists pinf, gamma, mu,
    # rho0, p0 (u0, v0, w0 optional, >= 0 as m5_input.c:113-135 checks them)
    m5: dict | None = None
    # refinement criteria of tag passes on the final state (harness .tag file), one tuple
    # per pass: (uniform, lvl, prs, lvl, thr, rho, lvl, thr, vel, lvl, thr, inter0, lvl,
    # lrs, inter1, lvl, lrs) as the reference's input file gives them
    tags: tuple | None = None
    # criteria of the reference's own meshadaptation run on the final state (harness
    # .adapt file); the adapted leaf list comes back as the third dump
    adapt: tuple | None = None
    # write the reference's own restart file of the final state (restart_save.c)
    restart: bool = False

    @property
    def neq(self) -> int:
        return 5 if self.model == 0 else 3 * len(self.m5["gamma"]) + 12


def _ct_lines(c: Case, levels: int) -> list[str]:
    lv = max(levels, 1)
    L = [
        f"MODEL\t{c.model}", "TYPE_INIT\t0", "VERBOSE\t0", "CASE\t1", "NS\t0", "NBCOMMS\t0",
        f"ORDER\t{c.order}", "GRAD_SCHEME\t1", "PRIMTV\t0", "LIMITER\t0",
        f"RK_STEPS\t{c.rk_steps}", f"DT\t{c.dt:.17e}", f"NSTEP\t{c.steps - 1}",
        "EXPORT_TYPE\t0", "EXPORT_STEP\t1000000", "RESTART_STEP\t1000000", "ADAPTH\t0",
        "ADAPTHSTEP\t1000", "GEO_ADAPTH\t1",
        f"CRT_UNIFORM\t1\t{lv}", f"CRT_GEO_AREA\t0\t0", "CRT_GRAD_PRS\t0\t0\t0.0",
        "CRT_GRAD_RHO\t0\t0\t0.0", "CRT_GRAD_VEL\t0\t0\t0.0",
        "RESTART\t0", "TRANSLATOR\t0", "MSCALE\t1.0", "SPLITMODE\t8",
        "NXQUAD\t0.0", "NYQUAD\t0.0", "NZQUAD\t0.0", "ZEROU0\t0", "ZEROU1\t0", "ZEROU2\t0",
        "BCOVERWRT\t0\t0\t0\t0\t0\t0",
    ]
    return L


def write_case(c: Case, d: str, name: str = "case") -> str:
    tx, ty, tz = c.trees
    base = os.path.join(d, name)
    nx, ny, nz = tx + 1, ty + 1, tz + 1

    def nid(i, j, k):
        return 1 + i + nx * (j + ny * k)

    with open(base + ".nd", "w") as f:
        f.write(f"{nx * ny * nz} \n")
        for k in range(nz):
            for j in range(ny):
                for i in range(nx):
                    f.write(f"{nid(i, j, k)}\t{i / tx:.17e}\t{j / ty:.17e}\t{k / tz:.17e}\n")
    nbits = max(tx, ty, tz).bit_length()
    trees = sorted(((i, j, k) for k in range(tz) for j in range(ty) for i in range(tx)),
                   key=lambda t: morton_key(*t, nbits, c.layout))
    bcfaces = {1: [], 2: [], 3: [], 4: []}
    with open(base + ".el", "w") as f:
        f.write(f"{len(trees)} \n")
        for e, (i, j, k) in enumerate(trees):
            nodes = []
            for q in range(8):
                cx, cy, cz = corner_xyz(q, c.layout)
                nodes.append(nid(i + cx, j + cy, k + cz))
            f.write(f"{e + 1}\t4\t" + "\t".join(str(n) for n in nodes) + "\n")
            for fc in range(6):
                pts = [corner_xyz(q, c.layout) for q in FACE_NODES[fc]]
                for ax, (lo, hi) in enumerate(((i, tx), (j, ty), (k, tz))):
                    vals = {p[ax] for p in pts}
                    if len(vals) == 1:
                        v = vals.pop()
                        side = None
                        if v == 0 and (i, j, k)[ax] == 0:
                            side = 2 * ax
                        if v == 1 and (i, j, k)[ax] == hi - 1:
                            side = 2 * ax + 1
                        if side is not None:
                            code = c.bc[side]
                            if code not in bcfaces:
                                raise ValueError("bc codes 1..4 only")
                            bcfaces[code].append((e + 1, fc + 1))
    for code, ext in zip((1, 2, 3, 4), (".ba", ".bb", ".bc", ".bd")):
        with open(base + ext, "w") as f:
            f.write(f"{len(bcfaces[code])}\n")
            for e, fc in bcfaces[code]:
                f.write(f"{e}\t{fc}\n")
    levels = c.level
    if c.refine:
        toks = c.refine.split()
        levels = max(levels, max(int(float(t)) for t in toks[-2:]))
    with open(base + ".ct", "w") as f:
        f.write("\n".join(_ct_lines(c, levels)) + "\n")
        if c.model == 5:
            q = c.m5
            nm = len(q["gamma"])

            def row(name, vals):
                return name + "".join(f"\t{v:.17e}" for v in vals) + "\n"

            f.write(f"AVF_LIM\t{q['avf_lim']:.17e}\nPRELAX\t{q['prelax']}\n")
            f.write(f"NMATERIALS\t{nm}\nAMIN\t{q['amin']:.17e}\n")
            f.write("CRT_ADAPT_INTER_0\t0\t0\t0\nCRT_ADAPT_INTER_1\t0\t0\t0\n")
            f.write(row("P_INF", q["pinf"]) + row("GAMMA", q["gamma"]) + row("MU", q["mu"]))
            f.write(row("VISC", [0.0] * nm) + row("RHO_INIT", q["rho0"]) + row("PR_INIT", q["p0"]))
            for key in ("u0", "v0", "w0"):
                f.write(row(key.upper(), q.get(key, [0.0] * nm)))
    if c.model == 0:
        with open(base + ".m0ct", "w") as f:
            f.write("".join(f"SKIP{i}\t0\n" for i in range(31)))
            f.write(f"MATERPINF\t{c.pinf:.17e}\nMATERGAMA\t{c.gamma:.17e}\nMATERVISC\t0.0\n")
    with open(base + ".ic", "w") as f:
        f.write(c.ic + "\n")
    if c.refine:
        with open(base + ".rf", "w") as f:
            f.write(c.refine + "\n")
    if c.tags is not None:
        with open(base + ".tag", "w") as f:
            for t in c.tags:
                f.write(" ".join(repr(float(v)) if isinstance(v, float) else str(int(v))
                                 for v in t) + "\n")
    if c.restart:
        with open(base + ".restart", "w") as f:
            f.write("1\n")
    if c.adapt is not None:
        with open(base + ".adapt", "w") as f:
            f.write(" ".join(repr(float(v)) if isinstance(v, float) else str(int(v))
                             for v in c.adapt) + "\n")
    if c.m5 and c.m5.get("mix"):
        with open(base + ".mix", "w") as f:
            f.write(c.m5["mix"] + "\n")
    return base


@dataclass
class Dump:
    model: int
    neq: int
    n: int
    loop_seconds: float
    steps: int
    root: np.ndarray
    level: np.ndarray
    adrs: np.ndarray
    xc: np.ndarray
    vol: np.ndarray
    si: np.ndarray
    bc: np.ndarray
    nneig: np.ndarray
    nsfc: np.ndarray
    neigfc: np.ndarray
    nb: np.ndarray
    area: np.ndarray
    normals: np.ndarray
    dist_cf: np.ndarray
    dist_cc: np.ndarray
    S: np.ndarray
    tags: np.ndarray | None = None  # [npass, n, 4]: SI[0], SI[1], split, smoothed split
    adapted: "Dump | None" = None  # the leaf list after the reference's meshadaptation
    restart_text: str | None = None  # the reference's restart file of this state


_LEAF_HDR = struct.Struct("<2i16i3dd2i")
_FACE = struct.Struct("<4i4i4d9d2d")


def read_dump(path: str) -> Dump:
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != b"FFVD":
        raise ValueError("not a dump")
    ver, model, neq, n = struct.unpack_from("<4i", buf, 4)
    loop_s, = struct.unpack_from("<d", buf, 20)
    steps, = struct.unpack_from("<q", buf, 28)
    off = 36
    rec = _LEAF_HDR.size + 6 * _FACE.size + 8 * neq
    dt = np.dtype([
        ("root", "<i4"), ("level", "<i4"), ("adrs", "<i4", 16), ("xc", "<f8", 3), ("vol", "<f8"),
        ("si", "<i4", 2),
        ("faces", [("bc", "<i4"), ("nn", "<i4"), ("nsfc", "<i4"), ("neigfc", "<i4"),
                   ("nb", "<i4", 4), ("area", "<f8", 4), ("nrm", "<f8", 9), ("dcf", "<f8"),
                   ("dcc", "<f8")], 6),
        ("S", "<f8", neq),
    ])
    assert dt.itemsize == rec, (dt.itemsize, rec)
    a = np.frombuffer(buf, dtype=dt, count=n, offset=off)
    fc = a["faces"]
    return Dump(model, neq, n, loop_s, steps, a["root"].copy(), a["level"].copy(),
                a["adrs"].copy(), a["xc"].copy(), a["vol"].copy(), a["si"].copy(),
                fc["bc"].copy(), fc["nn"].copy(), fc["nsfc"].copy(), fc["neigfc"].copy(),
                fc["nb"].copy(), fc["area"].copy(), fc["nrm"].copy(), fc["dcf"].copy(),
                fc["dcc"].copy(), a["S"].copy())


def run_case(c: Case, workdir: str | None = None, timeout: float = 600.0):
    """Run the reference on `c`; returns (init Dump, final Dump, stdout)."""
    if not ref_available():
        raise RuntimeError("reference oracle binary not built (oracle/_ref/forestfv_ref)")
    own = workdir is None
    d = workdir or tempfile.mkdtemp(prefix="ffvref_")
    try:
        base = write_case(c, d)
        run = os.path.join(d, "run")
        r = subprocess.run([REF_BIN, base, run], capture_output=True, text=True, timeout=timeout,
                           cwd=d)
        if r.returncode != 0 or not os.path.exists(run + ".final.bin"):
            raise RuntimeError(f"reference run failed rc={r.returncode}\n{r.stdout[-3000:]}\n"
                               f"{r.stderr[-3000:]}")
        final = read_dump(run + ".final.bin")
        if os.path.exists(run + ".tags.bin"):
            with open(run + ".tags.bin", "rb") as f:
                buf = f.read()
            assert buf[:4] == b"FFVT"
            npass, n = struct.unpack_from("<2i", buf, 4)
            final.tags = np.frombuffer(buf, dtype="<i4", count=4 * n * npass,
                                       offset=12).reshape(npass, n, 4).copy()
        if os.path.exists(run + ".adapt.bin"):
            final.adapted = read_dump(run + ".adapt.bin")
        rs = sorted(x for x in os.listdir(d) if x.startswith("restart") and x.endswith(".dat"))
        if rs:
            with open(os.path.join(d, rs[-1])) as f:
                final.restart_text = f.read()
        return read_dump(run + ".init.bin"), final, r.stdout
    finally:
        if own:
            import shutil
            shutil.rmtree(d, ignore_errors=True)
