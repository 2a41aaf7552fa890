"""Scene files and state dumps in the format of the reference's parity
harness, so that scenes move between this backend, the reference's CPU
engine and its upstream C++ solver unchanged.

`.scene` text (test/parity/scene_loader.mjs:20-84, the same records as
test/parity/reference_main.cpp:45-129): one record per line, `#` starts a
comment, tokens are separated by blanks, `inf` / `-inf` are infinities.

    body   sx sy sz density friction px py pz vx vy vz qx qy qz qw wx wy wz
    joint  ia ib rax ray raz rbx rby rbz stiffnessLin stiffnessAng fracture
    spring ia ib rax ray raz rbx rby rbz stiffness rest

A body record is the reference's legacy box constructor (`new Rigid(solver,
size, density, friction, position, velocity)`, src/physics/rigid.js:29-95:
mass = sx sy sz density, so density 0 makes it static) followed by its
orientation and angular velocity. Bodies are numbered in record order; a
joint with ia < 0 anchors r_a in the world. Joints and springs enter the
force list in record order (the Gauss-Seidel sweep depends on it). A spring
record's rest length is used as given (the loaders pass it straight to the
Spring constructor).

State dump (test/parity/reference_main.cpp:132-145): after each step one line
per body, `step index px py pz qx qy qz qw vx vy vz wx wy wz`, every number
printed with %.17g (the shortest form that round-trips a double exactly).
"""
from __future__ import annotations

import math

import numpy as np

from .abi import World
from .scene import INF, SHAPE_SPHERE, Scene

BODY_FIELDS = 18
JOINT_FIELDS = 11
SPRING_FIELDS = 10


class SceneFormatError(ValueError):
    pass


def _value(tok: str) -> float:
    """parseValue of both loaders: inf / -inf, else a decimal number."""
    if tok == "inf":
        return math.inf
    if tok == "-inf":
        return -math.inf
    try:
        return float(tok)
    except ValueError as e:
        raise SceneFormatError(f"not a number: {tok!r}") from e


def _index(tok: str) -> int:
    v = _value(tok)
    if not math.isfinite(v) or v != int(v):
        raise SceneFormatError(f"not a body index: {tok!r}")
    return int(v)


def parse_scene(text: str, name: str = "scene") -> Scene:
    """Bodies, joints and springs of a `.scene` text, in record order."""
    s = Scene(name)
    s.density = []
    for lineno, raw in enumerate(text.splitlines(), 1):
        tok = raw.split("#", 1)[0].split()
        if not tok:
            continue
        kind, args = tok[0], tok[1:]
        if kind == "body":
            if len(args) < BODY_FIELDS:
                raise SceneFormatError(f"line {lineno}: a body needs {BODY_FIELDS} values")
            v = [_value(t) for t in args[:BODY_FIELDS]]
            s.box(v[0:3], v[3], v[4], v[5:8], v[8:11], quat=tuple(v[11:15]), omega=tuple(v[15:18]))
            s.density.append(v[3])
        elif kind in ("joint", "spring"):
            need = JOINT_FIELDS if kind == "joint" else SPRING_FIELDS
            if len(args) < need:
                raise SceneFormatError(f"line {lineno}: a {kind} needs {need} values")
            ia, ib = _index(args[0]), _index(args[1])
            v = [_value(t) for t in args[2:need]]
            lo = -1 if kind == "joint" else 0
            if not (lo <= ia < s.n) or not (0 <= ib < s.n):
                raise SceneFormatError(f"line {lineno}: {kind} names a body not defined before it")
            if kind == "joint":
                s.joint(ia, ib, v[0:3], v[3:6], v[6], v[7], v[8])
            else:
                if not v[7] >= 0:
                    raise SceneFormatError(f"line {lineno}: spring rest length {v[7]} (must be >= 0)")
                s.spring(ia, ib, v[0:3], v[3:6], v[6], v[7])
        else:
            raise SceneFormatError(f"line {lineno}: unknown record: {kind}")
    return s


def load_scene(path: str) -> Scene:
    with open(path) as f:
        text = f.read()
    import os

    return parse_scene(text, os.path.splitext(os.path.basename(path))[0])


def _g(x: float) -> str:
    return "%.17g" % x


def _density(s: Scene, i: int) -> float:
    dens = getattr(s, "density", None)
    if dens is not None and i < len(dens):
        return dens[i]
    sx, sy, sz = s.b["size"][i]
    m = s.b["mass"][i]
    if m == 0:
        return 0.0
    d = m / (sx * sy * sz)
    if sx * sy * sz * d != m:
        raise SceneFormatError(f"body {i}: its mass is not size x density for any double density")
    return d


def format_scene(s: Scene) -> str:
    """The `.scene` text of `s` (boxes only: the format's body record is the
    box constructor). Every number with %.17g, so parsing gives `s` back bit
    for bit. Joints and springs are written in their force-list order."""
    lines = [f"# scene: {s.name}"]
    for i in range(s.n):
        if s.b["shape"][i] == SHAPE_SPHERE:
            raise SceneFormatError(f"body {i} is a sphere; .scene body records are boxes")
        v = (list(s.b["size"][i]) + [_density(s, i), s.b["friction"][i]] + list(s.b["pos"][i])
             + list(s.b["vel"][i]) + list(s.b["quat"][i]) + list(s.b["omega"][i]))
        lines.append("body " + " ".join(_g(x) for x in v))
    forces = [(j[7], "joint", j) for j in s.joints] + [(sp[7], "spring", sp) for sp in s.springs]
    for _, kind, f in sorted(forces, key=lambda t: t[0]):
        a, b, ra, rb = f[0], f[1], f[2], f[3]
        rest = [f[4], f[5], f[6]] if kind == "joint" else [f[4], f[5]]
        lines.append(f"{kind} {int(a)} {int(b)} " + " ".join(_g(x) for x in list(ra) + list(rb) + rest))
    return "\n".join(lines) + "\n"


def save_scene(s: Scene, path: str):
    with open(path, "w") as f:
        f.write(format_scene(s))


def format_state(w: World, step: int) -> str:
    """The dump lines of one step: `step index p(3) q(4) v(3) w(3)`, %.17g."""
    out = []
    for i in range(w.n_bodies):
        v = list(w.pos[i]) + list(w.quat[i]) + list(w.vel[i]) + list(w.omega[i])
        out.append(f"{step} {i} " + " ".join(_g(float(x)) for x in v))
    return "\n".join(out) + ("\n" if out else "")


def parse_states(text: str) -> dict:
    """Dump text -> {step: array (bodies, 13): p, q, v, w}; the body index
    column must count 0, 1, ... within each step."""
    rows: dict[int, list] = {}
    for lineno, raw in enumerate(text.splitlines(), 1):
        tok = raw.split()
        if not tok:
            continue
        if len(tok) != 15:
            raise SceneFormatError(f"line {lineno}: a state line has 15 fields, not {len(tok)}")
        step, idx = int(tok[0]), int(tok[1])
        r = rows.setdefault(step, [])
        if idx != len(r):
            raise SceneFormatError(f"line {lineno}: body {idx} out of order in step {step}")
        r.append([_value(t) for t in tok[2:]])
    return {k: np.array(v, dtype=np.float64) for k, v in rows.items()}


def state_array(w: World) -> np.ndarray:
    """The dump's 13 columns of a world's bodies (for comparisons)."""
    return np.concatenate([w.pos, w.quat, w.vel, w.omega], axis=1)


__all__ = ["parse_scene", "load_scene", "format_scene", "save_scene", "format_state", "parse_states",
           "state_array", "SceneFormatError", "INF"]
