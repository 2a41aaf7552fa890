"""Scene construction mirroring the reference scene graph.

`Scene.box` / `Scene.sphere` / `Scene.joint` / `Scene.spring` compute the same
derived quantities, with the same f64 operation order, as the reference
constructors:

  box     `new Rigid(...)`   src/physics/rigid.js:29-98  (mass, moments, radius)
  sphere  `Rigid.sphere`     src/physics/rigid.js:105-133
  joint   `new Joint(...)`   src/physics/joint.js:74-113
  spring  `new Spring(...)`  src/physics/spring.js:414-444 (rest < 0 = current length)

Bodies, joints and springs keep creation order, which the reference's
Gauss-Seidel order depends on (src/physics/solver.js:35-38). `Scene.world()`
returns an `abi.World` (numpy SoA) for the CUDA backend and the oracle.

The preset builders at the bottom are the benchmark and parity workloads:
the 10-cube stack, the 51,039-box pyramid with a falling sphere, the heavy
chain + spring chain, the batch of random piles, the bonded brick wall, and a
set of small parity scenes with the same content as the reference's parity
scene list (test/parity/gen_scenes.mjs).
"""
from __future__ import annotations

import math

import numpy as np

from .abi import SHAPE_BOX, SHAPE_SPHERE, World

INF = math.inf


def _rotate(q, v):
    """quat.rotateVec (src/math/maths.js:599-613), f64, same term order."""
    ux, uy, uz, w = q
    vx, vy, vz = v
    tx = (uy * vz - uz * vy) * 2
    ty = (uz * vx - ux * vz) * 2
    tz = (ux * vy - uy * vx) * 2
    return (vx + tx * w + (uy * tz - uz * ty),
            vy + ty * w + (uz * tx - ux * tz),
            vz + tz * w + (ux * ty - uy * tx))


def axis_angle(axis, angle):
    """Unit quaternion for a rotation of `angle` about `axis` (normalised here,
    as `Rigid.setOrientation` does, src/physics/rigid.js:262-267)."""
    ax, ay, az = axis
    n = math.sqrt(ax * ax + ay * ay + az * az) or 1.0
    h = angle * 0.5
    s = math.sin(h)
    return (ax / n * s, ay / n * s, az / n * s, math.cos(h))


class LCG:
    """The scene library's seeded PRNG (src/app/scenes.js:78-84)."""

    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFF

    def __call__(self) -> float:
        self.s = (self.s * 1664525 + 1013904223) & 0xFFFFFFFF
        return self.s / 4294967296.0

    def uniform(self, lo, hi):
        return lo + (hi - lo) * self()

    def log_uniform(self, lo, hi):
        return math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * self())


class Scene:
    def __init__(self, name: str = "scene"):
        self.name = name
        self.b = {k: [] for k in ("shape", "size", "mass", "moment", "radius", "friction", "pos",
                                  "quat", "vel", "omega")}
        self.joints = []
        self.springs = []
        self.params = {}
        self.meta = {}

    # --- bodies -------------------------------------------------------------
    @property
    def n(self):
        return len(self.b["mass"])

    def box(self, size, density, friction, position, velocity=(0.0, 0.0, 0.0), quat=None, omega=None):
        sx, sy, sz = (float(v) for v in size)
        mass = sx * sy * sz * density
        moment = (((sy * sy + sz * sz) / 12.0) * mass,
                  ((sx * sx + sz * sz) / 12.0) * mass,
                  ((sx * sx + sy * sy) / 12.0) * mass)
        hx, hy, hz = sx * 0.5, sy * 0.5, sz * 0.5
        radius = math.sqrt(hx * hx + hy * hy + hz * hz)
        return self._add(SHAPE_BOX, (sx, sy, sz), mass, moment, radius, friction, position, velocity,
                         quat, omega)

    def sphere(self, diameter, density, friction, position, velocity=(0.0, 0.0, 0.0), quat=None, omega=None):
        if not (math.isfinite(diameter) and diameter > 0):
            raise ValueError("sphere diameter must be a finite positive number")
        radius = diameter * 0.5
        mass = (4 / 3) * math.pi * radius * radius * radius * density
        inertia = (2 / 5) * mass * radius * radius
        return self._add(SHAPE_SPHERE, (diameter, diameter, diameter), mass, (inertia,) * 3, radius,
                         friction, position, velocity, quat, omega)

    def _add(self, shape, size, mass, moment, radius, friction, position, velocity, quat, omega):
        b = self.b
        b["shape"].append(shape)
        b["size"].append(tuple(size))
        b["mass"].append(float(mass))
        b["moment"].append(tuple(moment))
        b["radius"].append(float(radius))
        b["friction"].append(float(friction))
        b["pos"].append(tuple(float(v) for v in position))
        b["quat"].append(tuple(quat) if quat is not None else (0.0, 0.0, 0.0, 1.0))
        b["vel"].append(tuple(float(v) for v in velocity))
        b["omega"].append(tuple(omega) if omega is not None else (0.0, 0.0, 0.0))
        return self.n - 1

    def set_orientation(self, i, axis, angle):
        self.b["quat"][i] = axis_angle(axis, angle)

    # --- forces -------------------------------------------------------------
    def joint(self, a, b, r_a, r_b, stiffness_lin=INF, stiffness_ang=0.0, fracture=INF):
        self.joints.append((a, b, tuple(r_a), tuple(r_b), stiffness_lin, stiffness_ang, fracture,
                            len(self.joints) + len(self.springs)))
        return len(self.joints) - 1

    def spring(self, a, b, r_a, r_b, stiffness, rest=-1.0, tear_strain=INF):
        if rest < 0:
            pa = self._world_point(a, r_a)
            pb = self._world_point(b, r_b)
            d = (pa[0] - pb[0], pa[1] - pb[1], pa[2] - pb[2])
            rest = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
        self.springs.append((a, b, tuple(r_a), tuple(r_b), stiffness, rest, tear_strain,
                             len(self.joints) + len(self.springs)))
        return len(self.springs) - 1

    def _world_point(self, i, local):
        r = _rotate(self.b["quat"][i], local)
        p = self.b["pos"][i]
        return (r[0] + p[0], r[1] + p[1], r[2] + p[2])

    # --- export -------------------------------------------------------------
    def world(self) -> World:
        w = World(self.n, len(self.joints), len(self.springs))
        b = self.b
        w.shape[:] = b["shape"]
        w.size[:] = b["size"]
        w.mass[:] = b["mass"]
        w.moment[:] = b["moment"]
        w.radius[:] = b["radius"]
        w.friction[:] = b["friction"]
        w.pos[:] = b["pos"]
        w.quat[:] = b["quat"]
        w.vel[:] = b["vel"]
        w.omega[:] = b["omega"]
        w.prev_vel[:] = w.vel  # rigid.js:51
        for j, (a, bb, ra, rb, kl, ka, fr, order) in enumerate(self.joints):
            w.j_body_a[j], w.j_body_b[j] = a, bb
            w.j_r_a[j], w.j_r_b[j] = ra, rb
            w.j_stiffness_lin[j], w.j_stiffness_ang[j], w.j_fracture[j] = kl, ka, fr
            w.j_order[j] = order
        for s, (a, bb, ra, rb, k, rest, tear, order) in enumerate(self.springs):
            w.s_body_a[s], w.s_body_b[s] = a, bb
            w.s_r_a[s], w.s_r_b[s] = ra, rb
            w.s_stiffness[s], w.s_rest[s], w.s_tear_strain[s] = k, rest, tear
            w.s_order[s] = order
        return w


def add_ground(scene: Scene, friction=0.5):
    """A 400x400x4 static box whose top face is z = 0 (src/app/scenes.js:97-103)."""
    t = 4.0
    return scene.box((400.0, 400.0, t), 0.0, friction, (0.0, 0.0, -t / 2))


def batch_worlds(worlds):
    """Concatenate independent scenes into one batched world."""
    nb = [w.n_bodies for w in worlds]
    starts = np.concatenate([[0], np.cumsum(nb)]).astype(np.int32)
    nj = sum(w.n_joints for w in worlds)
    ns = sum(w.n_springs for w in worlds)
    out = World(int(starts[-1]), nj, ns, scene_start=starts)
    for f in ("shape", "size", "mass", "moment", "radius", "friction", "pos", "quat", "vel", "omega",
              "prev_vel"):
        setattr(out, f, np.ascontiguousarray(np.concatenate([getattr(w, f) for w in worlds])))
    jo = so = 0
    for w, s0 in zip(worlds, starts[:-1]):
        for f in ("j_r_a", "j_r_b", "j_stiffness_lin", "j_stiffness_ang", "j_fracture", "j_penalty_lin",
                  "j_penalty_ang", "j_lambda_lin", "j_lambda_ang", "j_broken"):
            getattr(out, f)[jo:jo + w.n_joints] = getattr(w, f)
        out.j_body_a[jo:jo + w.n_joints] = np.where(w.j_body_a < 0, -1, w.j_body_a + s0)
        out.j_body_b[jo:jo + w.n_joints] = w.j_body_b + s0
        out.j_order[jo:jo + w.n_joints] = w.j_order + jo + so
        for f in ("s_r_a", "s_r_b", "s_stiffness", "s_rest", "s_tear_strain", "s_penalty", "s_peak_strain",
                  "s_broken"):
            getattr(out, f)[so:so + w.n_springs] = getattr(w, f)
        out.s_body_a[so:so + w.n_springs] = w.s_body_a + s0
        out.s_body_b[so:so + w.n_springs] = w.s_body_b + s0
        out.s_order[so:so + w.n_springs] = w.s_order + jo + so
        jo += w.n_joints
        so += w.n_springs
    return out


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------

def cube_stack(n=10, seed=1, beta=10.0, gravity=-9.81):
    """Ten 1 m cubes (1000 kg/m^3, mu 0.5) stacked on the ground, each with a
    seeded +-0.01 m xy jitter and +-2 degree yaw about z. `beta` is the
    penalty ramp of both rows; None keeps the reference's own ramps (betaLin
    1e4, betaAng 100, src/physics/solver.js:97-104). With beta = 10 the ramp
    cannot stiffen the contacts of 1000 kg cubes within a step and the stack
    sinks through the ground, in the reference engine as on the device."""
    s = Scene("cube_stack")
    add_ground(s, 0.5)
    rnd = LCG(seed)
    for i in range(n):
        jx = rnd.uniform(-0.01, 0.01)
        jy = rnd.uniform(-0.01, 0.01)
        yaw = math.radians(rnd.uniform(-2.0, 2.0))
        k = s.box((1.0, 1.0, 1.0), 1000.0, 0.5, (jx, jy, 0.5 + i * 1.0))
        s.set_orientation(k, (0.0, 0.0, 1.0), yaw)
    s.params = dict(gravity=gravity, iterations=10, alpha=0.95)
    if beta is not None:
        s.params.update(beta_lin=beta, beta_ang=beta)
    s.meta = dict(steps=300)
    return s


def pyramid(layers=53, size=1.0, gap=0.01, density=1000.0, friction=0.6, sphere_radius=2.0,
            sphere_density=5000.0, sphere_speed=10.0, gravity=-9.81):
    """Square pyramid of `layers` layers (layer k from the top is a k x k grid
    of cubes; 51,039 cubes at 53 layers) with a 1% gap between neighbours, and
    a sphere dropped onto the apex. Ground, cubes, then the sphere."""
    s = Scene("pyramid")
    add_ground(s, friction)
    pitch = size * (1.0 + gap)
    n = layers
    shape, sizes, mass, moment, radius, fric, pos = [], [], [], [], [], [], []
    for layer in range(n):
        w = n - layer
        off = ((w - 1) * pitch) / 2
        xs = np.arange(w) * pitch - off
        gx, gy = np.meshgrid(xs, xs, indexing="ij")
        z = layer * pitch + size / 2
        p = np.stack([gx.ravel(), gy.ravel(), np.full(w * w, z)], axis=1)
        pos.append(p)
    pos = np.concatenate(pos)
    m = len(pos)
    base = s.n
    # Vectorised `new Rigid(...)` for identical cubes (rigid.js:72-88)
    sx = sy = sz = float(size)
    cube_mass = sx * sy * sz * density
    cube_moment = (((sy * sy + sz * sz) / 12.0) * cube_mass,) * 3
    hx = sx * 0.5
    cube_radius = math.sqrt(hx * hx + hx * hx + hx * hx)
    s.b["shape"].extend([SHAPE_BOX] * m)
    s.b["size"].extend([(sx, sy, sz)] * m)
    s.b["mass"].extend([cube_mass] * m)
    s.b["moment"].extend([cube_moment] * m)
    s.b["radius"].extend([cube_radius] * m)
    s.b["friction"].extend([float(friction)] * m)
    s.b["pos"].extend(map(tuple, pos.tolist()))
    s.b["quat"].extend([(0.0, 0.0, 0.0, 1.0)] * m)
    s.b["vel"].extend([(0.0, 0.0, 0.0)] * m)
    s.b["omega"].extend([(0.0, 0.0, 0.0)] * m)
    apex_top = (n - 1) * pitch + size
    s.sphere(2 * sphere_radius, sphere_density, friction, (0.0, 0.0, apex_top + sphere_radius + 1.0),
             (0.0, 0.0, -sphere_speed))
    s.params = dict(gravity=gravity, iterations=10)
    s.meta = dict(steps=600, cubes=m, first_cube=base)
    return s


def heavy_chain(links=50, end_mass=26000.0, springs=100, gravity=-9.81):
    """A 50-link chain of hard ball sockets (0.2 x 0.2 x 1.0 m links of 1 kg)
    hung from a world anchor and ending in a 26,000 kg box, released 40
    degrees off vertical; beside it a 100-spring chain of 1 kg bodies with
    stiffness alternating 1e3 / 1e6 N/m, built at its analytic equilibrium."""
    s = Scene("heavy_chain")
    add_ground(s, 0.5)
    L = 1.0
    top = (0.0, 0.0, 80.0)
    ang = math.radians(40.0)
    q = axis_angle((0.0, 1.0, 0.0), ang)
    along = lambda d: (top[0] - math.sin(ang) * d, top[1], top[2] - math.cos(ang) * d)
    link_density = 1.0 / (0.2 * 0.2 * L)
    prev = None
    for i in range(links):
        b = s.box((0.2, 0.2, L), link_density, 0.4, along(i * L + L / 2), quat=q)
        if prev is None:
            s.joint(-1, b, top, (0.0, 0.0, L / 2))
        else:
            s.joint(prev, b, (0.0, 0.0, -L / 2), (0.0, 0.0, L / 2))
        prev = b
    E = 3.0
    end = s.box((E, E, E), end_mass / (E * E * E), 0.5, along(links * L + E / 2), quat=q)
    s.joint(prev, end, (0.0, 0.0, -L / 2), (0.0, 0.0, E / 2))
    # spring chain at its analytic equilibrium (the fixture of test/fixtures.mjs:62-135),
    # 150 m away: beyond the reach of the swinging chain (radius 53 m)
    g = abs(gravity)
    anchor = s.box((0.4, 0.4, 0.4), 0.0, 0.5, (150.0, 0.0, 150.0))
    prev = anchor
    z = 150.0
    size = 0.1
    for i in range(springs):
        k = 1e3 if i % 2 == 0 else 1e6
        ext = g * (springs - i) * 1.0 / k
        z -= 1.0 + ext
        b = s.box((size, size, size), 1.0 / (size * size * size), 0.5, (150.0, 0.0, z))
        s.spring(prev, b, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), k, 1.0)
        prev = b
    s.params = dict(gravity=gravity, iterations=20)
    s.meta = dict(steps=1000, end_body=end, chain_bodies=(0, end + 1))
    return s


def random_pile(n_bodies, seed, gravity=-9.81):
    """One scene of the batched workload: `n_bodies` boxes with edges
    U[0.3, 2.0] m, density log-uniform [100, 1e4] kg/m^3 and mu U[0.2, 0.9],
    placed on a contact-free lattice (pitch 3.5 m > any box diagonal) above
    the ground so the pile forms by falling."""
    s = Scene(f"pile{seed}")
    add_ground(s, 0.5)
    rnd = LCG(seed)
    side = max(1, int(math.ceil(n_bodies ** (1.0 / 3.0))))
    pitch = 3.5
    for i in range(n_bodies):
        ix, iy, iz = i % side, (i // side) % side, i // (side * side)
        size = (rnd.uniform(0.3, 2.0), rnd.uniform(0.3, 2.0), rnd.uniform(0.3, 2.0))
        density = rnd.log_uniform(100.0, 1e4)
        mu = rnd.uniform(0.2, 0.9)
        x = (ix - (side - 1) / 2) * pitch
        y = (iy - (side - 1) / 2) * pitch
        z = 2.0 + iz * pitch
        s.box(size, density, mu, (x, y, z))
    s.params = dict(gravity=gravity, iterations=10)
    s.meta = dict(steps=240)
    return s


def pile_batch(num_scenes=512, base_seed=1000, lo=64, hi=8192):
    """Scene sizes of the batched workload: log-uniform body counts in
    [lo, hi], one seed per scene (base + index)."""
    rnd = LCG(base_seed)
    counts = []
    for i in range(num_scenes):
        counts.append(int(round(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * rnd()))))
    return [random_pile(c, base_seed + 1 + i) for i, c in enumerate(counts)]


def brick_wall(cols=16, rows=16, fracture=500.0, sphere_mass=50.0, sphere_speed=8.0, gravity=-9.81):
    """A 16 x 16 wall of 0.5 x 0.25 x 0.25 m bricks bonded by hard ball
    sockets with hard angular rows and a fracture threshold, struck by a
    50 kg sphere."""
    s = Scene("brick_wall")
    add_ground(s, 0.5)
    bw, bd, bh = 0.5, 0.25, 0.25
    grid = [[None] * cols for _ in range(rows)]
    for r in range(rows):
        for c in range(cols):
            b = s.box((bw, bd, bh), 1000.0, 0.6, ((c - cols / 2) * bw, 0.0, bh / 2 + r * bh))
            grid[r][c] = b
            if c > 0:
                s.joint(grid[r][c - 1], b, (bw / 2, 0.0, 0.0), (-bw / 2, 0.0, 0.0), INF, INF, fracture)
            if r > 0:
                s.joint(grid[r - 1][c], b, (0.0, 0.0, bh / 2), (0.0, 0.0, -bh / 2), INF, INF, fracture)
    radius = 0.3
    density = sphere_mass / ((4 / 3) * math.pi * radius ** 3)
    s.sphere(2 * radius, density, 0.4, (0.0, -3.0, rows * bh * 0.5), (0.0, sphere_speed, 0.0))
    s.params = dict(gravity=gravity, iterations=10)
    s.meta = dict(steps=60)
    return s


def brick_wall_c5(mu=0.6, sphere_velocity=(0.0, 8.0, 0.0), bond_stiffness=INF, cols=16, rows=16,
                  sphere_mass=50.0, sphere_offset_z=0.1, gravity=-9.81):
    """The differentiable wall: 16 x 16 bricks of 0.5 x 0.25 x 0.25 m (density
    1000, friction `mu`) bonded by ball sockets with linear and angular rows of
    stiffness `bond_stiffness` (hard by default) and no fracture, and a 50 kg
    sphere of radius 0.3 m launched at `sphere_velocity`, its centre
    `sphere_offset_z` above the wall's mid-height. Choices that keep the
    objective differentiable in the f64 engine: the sphere off the seam between
    rows 7 and 8 (on it, the sign of the vertical velocity decides which row
    it strikes: a jump), and no fracture (a bond breaking is a jump). Finite
    bonds ramp their penalty by beta |C| towards the stiffness and, at the
    reference's ramp, never reach a cap of 1e4..1e6 within 60 steps while the
    wall sags, so the stiffness has no derivative there; hard bonds have no
    stiffness parameter (the penalty cap penalty_max stands in for it).
    Bodies: ground, bricks row by row, then the sphere."""
    s = Scene("brick_wall_c5")
    add_ground(s, 0.5)
    bw, bd, bh = 0.5, 0.25, 0.25
    grid = [[None] * cols for _ in range(rows)]
    k = float(bond_stiffness)
    for r in range(rows):
        for c in range(cols):
            b = s.box((bw, bd, bh), 1000.0, float(mu), ((c - cols / 2) * bw, 0.0, bh / 2 + r * bh))
            grid[r][c] = b
            if c > 0:
                s.joint(grid[r][c - 1], b, (bw / 2, 0.0, 0.0), (-bw / 2, 0.0, 0.0), k, k, INF)
            if r > 0:
                s.joint(grid[r - 1][c], b, (0.0, 0.0, bh / 2), (0.0, 0.0, -bh / 2), k, k, INF)
    radius = 0.3
    density = sphere_mass / ((4 / 3) * math.pi * radius ** 3)
    s.sphere(2 * radius, density, 0.4, (0.0, -3.0, rows * bh * 0.5 + sphere_offset_z),
             tuple(float(v) for v in sphere_velocity))
    s.params = dict(gravity=gravity, iterations=10)
    s.meta = dict(steps=60, bricks=(1, 1 + rows * cols))
    return s


def breakage(cols=6, rows=4, fracture=100.0, tear_strains=(0.02, 0.05), gravity=-9.81):
    """Constraints that break within the first steps: a `cols` x `rows` brick
    wall bonded by hard ball sockets with hard angular rows and a fracture
    threshold on |lambda_ang| (src/physics/joint.js:307-316), struck by a 50 kg
    sphere launched 0.8 m in front of it (bonds start breaking at step 4 in
    the f64 engine at fracture 100), and beside it one hanging chain of six
    1 kg boxes on springs (stiffness 1e3 / 1e4 alternating, rest 1 m) per
    entry of `tear_strains`, released at rest length so that the top spring
    overshoots its static strain and tears (src/physics/spring.js:461-470):
    at step 5 for 0.02, step 9 for 0.05."""
    s = brick_wall(cols=cols, rows=rows, fracture=fracture, gravity=gravity)
    s.name = "breakage"
    s.b["pos"][-1] = (0.0, -0.8, rows * 0.25 * 0.5)
    for c, tear in enumerate(tear_strains):
        x = 10.0 + 3.0 * c
        anchor = s.box((0.4, 0.4, 0.4), 0.0, 0.5, (x, 0.0, 20.0))
        prev, z = anchor, 20.0
        for i in range(6):
            z -= 1.0
            b = s.box((0.1, 0.1, 0.1), 1000.0, 0.5, (x, 0.0, z))
            s.spring(prev, b, (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 1e3 if i % 2 == 0 else 1e4, 1.0, tear)
            prev = b
    s.meta = dict(steps=15)
    return s


def joint_clique(n=72, stiffness=100.0, radius=6.0, gravity=-9.81):
    """A constraint graph that needs more colours than a body has contacts:
    `n` 1 kg boxes (0.3 m) on a horizontal circle, every pair joined by a
    finite ball socket (stiffness `stiffness`, no angular rows) anchored at
    the midpoint of the two centres, so every joint starts at C = 0. The
    graph is complete: any proper colouring needs n colours."""
    s = Scene("joint_clique")
    add_ground(s)
    ids, pos = [], []
    for k in range(n):
        a = 2.0 * math.pi * k / n
        p = (radius * math.cos(a), radius * math.sin(a), 10.0)
        ids.append(s.box((0.3, 0.3, 0.3), 1.0 / 0.027, 0.5, p))
        pos.append(p)
    for i in range(n):
        for j in range(i + 1, n):
            h = tuple((pos[j][k] - pos[i][k]) * 0.5 for k in range(3))
            s.joint(ids[i], ids[j], h, tuple(-x for x in h), stiffness, 0.0, INF)
    s.params = dict(gravity=gravity, iterations=10)
    s.meta = dict(steps=30)
    return s


def parity_scenes():
    """Small scenes with the content of the reference's parity list
    (test/parity/gen_scenes.mjs): ground, spinner, stack, stack_ratio,
    pyramid, rope, heavy_rope, rope_angular, static_friction, spring,
    spring_ratio, tumble. Gravity -10, the reference default."""
    out = []
    s = Scene("ground")
    s.box((100, 100, 1), 0, 0.5, (0, 0, 0))
    s.box((1, 1, 1), 1, 0.5, (0, 0, 4))
    out.append(s)

    s = Scene("spinner")
    s.box((2, 0.6, 1.4), 1, 0.5, (0, 0, 0), omega=(1.3, 2.1, -0.7))
    out.append(s)

    s = Scene("stack")
    s.box((100, 100, 1), 0, 0.5, (0, 0, 0))
    for i in range(10):
        s.box((1, 1, 1), 1, 0.5, (0, 0, i * 1.5 + 1.0))
    out.append(s)

    s = Scene("stack_ratio")
    s.box((100, 100, 1.0), 0, 0.5, (0, 0, 0))
    top, size = 0.5, 1.0
    for _ in range(4):
        half = size * 0.5
        cz = top + half
        s.box((size, size, size), 1, 0.5, (0, 0, cz))
        top = cz + half
        size *= 2.0
    out.append(s)

    s = Scene("pyramid")
    s.box((100, 100, 1), 0, 0.5, (0, 0, -0.5))
    S = 8
    for y in range(S):
        for x in range(S - y):
            s.box((1, 0.5, 0.5), 1, 0.5, (x * 1.01 + y * 0.5 - S / 2, 0, y * 0.85 + 0.5))
    out.append(s)

    def rope(name, n, last_size=None, angular=False):
        s = Scene(name)
        s.box((100, 100, 1), 0, 0.5, (0, 0, -20))
        prev = -1
        for i in range(n):
            last = last_size is not None and i == n - 1
            cur = s.box((last_size,) * 3 if last else (1, 0.5, 0.5), 0 if i == 0 else 1, 0.5,
                        (i + (last_size / 2 if last else 0), 0, 10))
            if prev >= 0:
                rb = (-last_size / 2, 0, 0) if last else (-0.5, 0, 0)
                s.joint(prev, cur, (0.5, 0, 0), rb, INF, INF if angular else 0.0)
            prev = cur
        return s

    out.append(rope("rope", 20))
    out.append(rope("heavy_rope", 20, last_size=5))
    out.append(rope("rope_angular", 12, angular=True))

    s = Scene("static_friction")
    s.box((100, 100, 1), 0, 0.5, (0, 0, 0))
    a = math.radians(30.0)
    q = (0.0, math.sin(a * 0.5), 0.0, math.cos(a * 0.5))
    s.box((40, 24, 1), 0, 1.0, (0, 0, 3), quat=q)
    tangent, normal = _rotate(q, (1, 0, 0)), _rotate(q, (0, 0, 1))
    for i in range(11):
        mu = (i / 10) * 0.25 + 0.25
        y = -10 + i * 2
        s.box((1, 1, 1), 1, mu, (tangent[0] * -12 + normal[0] * 1.05, tangent[1] * -12 + y + normal[1] * 1.05,
                                 3 + tangent[2] * -12 + normal[2] * 1.05))
    out.append(s)

    s = Scene("spring")
    s.box((100, 100, 1), 0, 0.5, (0, 0, 0))
    anchor = s.box((1, 1, 1), 0, 0.5, (0, 0, 14))
    block = s.box((2, 2, 2), 1, 0.5, (0, 0, 8))
    s.spring(anchor, block, (0, 0, 0), (0, 0, 0), 100, 4)
    out.append(s)

    s = Scene("spring_ratio")
    s.box((100, 100, 1), 0, 0.5, (0, 0, -10))
    prev, N = -1, 8
    for i in range(N):
        x = (i - (N - 1) * 0.5) * 3.0
        cur = s.box((1, 0.75, 0.75), 0 if i in (0, N - 1) else 1, 0.5, (x, 0, 12))
        if prev >= 0:
            s.spring(prev, cur, (0.5, 0, 0), (-0.5, 0, 0), 10 if i % 2 == 0 else 10000, 3)
        prev = cur
    out.append(s)

    s = Scene("tumble")
    s.box((100, 100, 1), 0, 0.5, (0, 0, 0))
    n = math.sqrt(0.3 * 0.3 + 0.8 * 0.8 + 0.5 * 0.5)
    for i in range(12):
        a = 0.3 + i * 0.37
        h = a * 0.5
        sn = math.sin(h)
        s.box((1.4, 0.8, 0.6), 1, 0.4, ((i % 3) * 1.3 - 1.3, (i // 3) * 1.3 - 1.3, 2 + i * 1.1),
              velocity=(0.4, -0.2, 0), quat=(0.3 / n * sn, 0.8 / n * sn, 0.5 / n * sn, math.cos(h)),
              omega=(0.5, -0.9, 0.3))
    out.append(s)
    return out


def spheres_scene():
    """Spheres resting, rolling and striking boxes: sphere-sphere and
    sphere-OBB manifolds with curved-basis warm start."""
    s = Scene("spheres")
    s.box((100, 100, 2), 0, 0.5, (0, 0, -1))
    s.sphere(1.0, 1.0, 0.5, (0, 0, 0.49), velocity=(2.0, 0, 0))
    s.sphere(1.0, 2.0, 0.5, (1.2, 0.3, 2.0))
    s.box((1, 1, 1), 1.0, 0.5, (-2.0, 0.0, 0.5))
    s.sphere(0.6, 1.0, 0.5, (-2.0, 0.1, 1.6), velocity=(0, 0, -1.0))
    s.box((1.2, 0.6, 0.8), 1.0, 0.5, (2.5, -1.5, 0.4))
    s.sphere(1.0, 1.0, 0.5, (1.25, -1.48, 0.5), velocity=(3.5, 0.6, 0), omega=(0, 0, 1.3))
    return s


def material_scene(kind="pile", seed=7):
    """Scenes for the WebGPU engine's contact extensions
    (AVBD_CONTACT_MATERIALS), with seeded per-body materials: static friction
    U[0.3, 0.9], dynamic friction a U[0.3, 1] fraction of it, restitution
    U[0, 0.8], rest offsets U[-0.02, -0.005] (the ground keeps the defaults).
    "pile": a 60-box random pile falling onto the ground; "drop": boxes and
    spheres thrown down onto the ground and each other fast enough to arm
    restitution; "spheres": spheres_scene. Returns (scene, materials dict for
    World.set_materials)."""
    if kind == "pile":
        s = random_pile(60, seed)
    elif kind == "drop":
        s = Scene("drop")
        add_ground(s, 0.6)
        rnd = LCG(seed)
        for i in range(12):
            x, y = (i % 4 - 1.5) * 1.6, (i // 4 - 1) * 1.6
            if i % 3 == 2:
                s.sphere(rnd.uniform(0.5, 1.0), 800.0, 0.6, (x, y, rnd.uniform(0.6, 1.2)),
                         velocity=(rnd.uniform(-0.5, 0.5), 0.0, -rnd.uniform(2.0, 4.0)))
            else:
                s.box((rnd.uniform(0.5, 1.0), rnd.uniform(0.5, 1.0), rnd.uniform(0.5, 1.0)), 600.0, 0.6,
                      (x, y, rnd.uniform(0.7, 1.3)), velocity=(rnd.uniform(-0.5, 0.5), 0.0, -rnd.uniform(2.0, 4.0)))
        s.params = dict(gravity=-9.81, iterations=10)
    elif kind == "spheres":
        s = spheres_scene()
        s.params = dict(gravity=-9.81, iterations=10)
    elif kind == "hover":
        # bodies starting a few millimetres apart, inside each other's contact
        # skin: speculative contacts from the first step
        s = Scene("hover")
        add_ground(s, 0.6)
        rnd = LCG(seed)
        for i in range(6):
            x = (i - 2.5) * 1.3
            s.box((1.0, 1.0, 0.5), 700.0, 0.6, (x, 0.0, 0.25 + rnd.uniform(0.001, 0.009)))
            s.box((0.6, 0.6, 0.6), 400.0, 0.6, (x, 0.0, 0.8 + rnd.uniform(0.0015, 0.009)),
                  velocity=(0.0, 0.0, -rnd.uniform(0.5, 1.5)))
        s.sphere(0.5, 900.0, 0.6, (4.5, 0.0, 0.25 + 0.004))
        s.params = dict(gravity=-9.81, iterations=10)
    else:
        raise KeyError(kind)
    rnd = LCG(seed * 7 + 3)
    n = s.n
    sf, df, e, ro = [], [], [], []
    for i in range(n):
        static = s.b["mass"][i] == 0
        a = rnd.uniform(0.3, 0.9)
        sf.append(s.b["friction"][i] if static else a)
        df.append(s.b["friction"][i] if static else a * rnd.uniform(0.3, 1.0))
        e.append(0.0 if static else rnd.uniform(0.0, 0.8))
        ro.append(-0.005 if static else rnd.uniform(-0.02, -0.005))
    return s, dict(static_friction=sf, dynamic_friction=df, restitution=e, rest_offset=ro)
