// cuda_backend.mjs - the CUDA backend as a third engine of the sandbox, with the
// method names of GpuBackend (src/physics/gpu/backend.js:243), so that the
// call sites of src/app/boot.js (:1798-1803, :2145-2150) can take it in place of
// the WebGPU backend. The solver's objects (Rigid, Joint, Spring; field names
// of src/physics/rigid.js:29-90, joint.js:74-113, spring.js:73-102) are packed
// into typed arrays for the addon (avbd_node.cc) and written back after reads,
// as syncToCPU does (backend.js:1984-2039).
import { createRequire } from 'node:module';

const require = createRequire(import.meta.url);
const addon = require('./build/Release/avbd_node.node');

const SHAPE_BOX = 0;
const SHAPE_SPHERE = 1;

const isJoint = (f) => f.stiffnessLin !== undefined && f.lambdaLin !== undefined;
const isSpring = (f) => f.tearStrain !== undefined && f.peakStrain !== undefined;

// The solver parameters avbd_create takes (Solver.defaultParams names).
const PARAM_NAMES = [
  'dt', 'gravity', 'iterations', 'postStabilize', 'betaLin', 'betaAng', 'alpha', 'gamma',
  'penaltyMin', 'penaltyMax', 'collisionMargin', 'stickThreshold', 'rotatedInertia',
  'springStiffnessRamp', 'springGeometricStiffness', 'cachedContactJacobians',
  'contactOffset', 'restOffset', 'restitutionThreshold', 'contactPersistence',
];

function paramsOf(solver, extra) {
  const p = {};
  for (const k of PARAM_NAMES) if (solver[k] !== undefined && solver[k] !== null) p[k] = solver[k];
  return Object.assign(p, extra);
}

function fill3(dst, i, v) { dst[i * 3] = v[0]; dst[i * 3 + 1] = v[1]; dst[i * 3 + 2] = v[2]; }
function read3(v, src, i) { v[0] = src[i * 3]; v[1] = src[i * 3 + 1]; v[2] = src[i * 3 + 2]; }

// Scene graph -> typed arrays (the layout of avbd_world), with the object ->
// index maps the write-back and the anchor updates use.
function toSoA(solver) {
  const bodies = solver.bodies;
  const n = bodies.length;
  const bodyIndex = new Map();
  const B = {
    count: n, shape: new Int32Array(n), size: new Float64Array(3 * n), mass: new Float64Array(n),
    moment: new Float64Array(3 * n), radius: new Float64Array(n), friction: new Float64Array(n),
    pos: new Float64Array(3 * n), quat: new Float64Array(4 * n), vel: new Float64Array(3 * n),
    omega: new Float64Array(3 * n), prevVel: new Float64Array(3 * n),
    // contact materials (rigid.js:54-68; read under contactModel 1)
    staticFriction: new Float64Array(n), dynamicFriction: new Float64Array(n), restitution: new Float64Array(n),
    contactOffset: new Float64Array(n), restOffset: new Float64Array(n),
  };
  bodies.forEach((b, i) => {
    bodyIndex.set(b, i);
    B.shape[i] = b.shape === 'sphere' ? SHAPE_SPHERE : SHAPE_BOX;
    fill3(B.size, i, b.size);
    B.mass[i] = b.mass;
    fill3(B.moment, i, b.moment);
    B.radius[i] = b.radius;
    B.friction[i] = b.friction;
    fill3(B.pos, i, b.positionLin);
    for (let c = 0; c < 4; c++) B.quat[i * 4 + c] = b.positionAng[c];
    fill3(B.vel, i, b.velocityLin);
    fill3(B.omega, i, b.velocityAng);
    fill3(B.prevVel, i, b.prevVelocityLin);
    B.staticFriction[i] = b.staticFriction ?? b.friction;
    B.dynamicFriction[i] = b.dynamicFriction ?? b.friction;
    B.restitution[i] = b.restitution ?? 0;
    // null offsets inherit the solver's (rigid.js:61-67)
    B.contactOffset[i] = b.contactOffset ?? solver.contactOffset ?? 0.005;
    B.restOffset[i] = b.restOffset ?? solver.restOffset ?? -0.005;
  });

  const joints = [];
  const springs = [];
  const jointOrder = [];
  const springOrder = [];
  solver.forces.forEach((f, k) => {
    // the app's drag joint stays CPU-side: the grab is uniform state here
    // (boot.js:606-611; the WebGPU pack skips it too, backend.js:945)
    if (f.isDragJoint) return;
    if (isJoint(f)) { joints.push(f); jointOrder.push(k); }
    else if (isSpring(f)) { springs.push(f); springOrder.push(k); }
  });
  const nj = joints.length;
  const jointIndex = new Map();
  const J = {
    count: nj, bodyA: new Int32Array(nj), bodyB: new Int32Array(nj), rA: new Float64Array(3 * nj),
    rB: new Float64Array(3 * nj), stiffnessLin: new Float64Array(nj), stiffnessAng: new Float64Array(nj),
    fracture: new Float64Array(nj), penaltyLin: new Float64Array(3 * nj), penaltyAng: new Float64Array(3 * nj),
    lambdaLin: new Float64Array(3 * nj), lambdaAng: new Float64Array(3 * nj), broken: new Int32Array(nj),
    order: Int32Array.from(jointOrder),
  };
  joints.forEach((j, i) => {
    jointIndex.set(j, i);
    J.bodyA[i] = j.bodyA ? bodyIndex.get(j.bodyA) : -1; // no body A: rA is a world point (drag joint)
    J.bodyB[i] = bodyIndex.get(j.bodyB);
    fill3(J.rA, i, j.rA);
    fill3(J.rB, i, j.rB);
    J.stiffnessLin[i] = j.stiffnessLin;
    J.stiffnessAng[i] = j.stiffnessAng;
    J.fracture[i] = j.fracture;
    fill3(J.penaltyLin, i, j.penaltyLin);
    fill3(J.penaltyAng, i, j.penaltyAng);
    fill3(J.lambdaLin, i, j.lambdaLin);
    fill3(J.lambdaAng, i, j.lambdaAng);
    J.broken[i] = j.broken ? 1 : 0;
  });

  const ns = springs.length;
  const springIndex = new Map();
  const S = {
    count: ns, bodyA: new Int32Array(ns), bodyB: new Int32Array(ns), rA: new Float64Array(3 * ns),
    rB: new Float64Array(3 * ns), stiffness: new Float64Array(ns), rest: new Float64Array(ns),
    tearStrain: new Float64Array(ns), penalty: new Float64Array(ns), peakStrain: new Float64Array(ns),
    broken: new Int32Array(ns), order: Int32Array.from(springOrder),
  };
  springs.forEach((s, i) => {
    springIndex.set(s, i);
    S.bodyA[i] = bodyIndex.get(s.bodyA);
    S.bodyB[i] = bodyIndex.get(s.bodyB);
    fill3(S.rA, i, s.rA);
    fill3(S.rB, i, s.rB);
    S.stiffness[i] = s.stiffness;
    S.rest[i] = s.rest;
    S.tearStrain[i] = s.tearStrain;
    S.penalty[i] = s.penalty;
    S.peakStrain[i] = s.peakStrain;
    S.broken[i] = s.broken ? 1 : 0;
  });
  return { world: { bodies: B, joints: J, springs: S }, bodyIndex, jointIndex, springIndex };
}

// Typed arrays -> scene graph: the fields syncToCPU writes (backend.js:2004-2035).
function fromSoA(solver, packed) {
  const { bodies: B, joints: J, springs: S } = packed.world;
  for (const [b, i] of packed.bodyIndex) {
    read3(b.positionLin, B.pos, i);
    for (let c = 0; c < 4; c++) b.positionAng[c] = B.quat[i * 4 + c];
    read3(b.velocityLin, B.vel, i);
    read3(b.velocityAng, B.omega, i);
    read3(b.prevVelocityLin, B.prevVel, i);
  }
  for (const [j, i] of packed.jointIndex) {
    read3(j.penaltyLin, J.penaltyLin, i);
    read3(j.penaltyAng, J.penaltyAng, i);
    read3(j.lambdaLin, J.lambdaLin, i);
    read3(j.lambdaAng, J.lambdaAng, i);
    if (J.broken[i]) j.broken = true;
  }
  for (const [s, i] of packed.springIndex) {
    s.penalty = S.penalty[i];
    s.peakStrain = S.peakStrain[i];
    s.broken = S.broken[i] !== 0;
  }
}

export class CudaBackend {
  constructor(options = {}) {
    // CUDA-only knobs: lanesPerBody, schedule, fp64RatioThreshold, waitLimit; contactModel: 1 selects the
    // WebGPU engine's contact extensions (materials, restitution, rest offsets)
    this.options = options;
    this.handle = null;
    this.paramsKey = '';
    this.packed = null;
    this.ready = false;
    this.topologyDirty = true;
    this.overrideColoring = null; // {colorOf: Int32Array, numColors}
    this.grab = null; // {body, local, target, stiffness} (backend.js:302-307), pushed every step
    this._profiling = false;
  }

  // GpuBackend.init (backend.js:337-450): nothing to compile; the context is
  // created at the first pack, with that solver's parameters.
  async init() { this.ready = true; return true; }

  // pack(solver) (backend.js:662): the whole scene; a new context when the
  // solver's parameters changed (they are fixed per context).
  pack(solver) {
    const params = paramsOf(solver, this.options);
    const key = JSON.stringify(params);
    if (!this.handle || key !== this.paramsKey) {
      if (this.handle) addon.destroy(this.handle);
      this.handle = addon.create(params);
      this.paramsKey = key;
      if (this._profiling) addon.setProfiling(this.handle, true);
    }
    const prev = this.packed && key === this.paramsKeyPacked ? this.packed : null;
    this.packed = toSoA(solver);
    if (prev) {
      // a topology edit: the live device state follows each Rigid, Joint and
      // Spring object to its new index (backend.js:662-1301, identity runs
      // :107-145), the warm-start contacts too when survivors keep their order
      const map = (items, index) => Int32Array.from(items, (x) => (index.has(x) ? index.get(x) : -1));
      const P = this.packed;
      const bodies = [...P.bodyIndex.keys()];
      const joints = [...P.jointIndex.keys()];
      const springs = [...P.springIndex.keys()];
      this.lastCarriedManifolds = addon.repack(this.handle, P.world, map(bodies, prev.bodyIndex),
        map(joints, prev.jointIndex), map(springs, prev.springIndex));
    } else {
      addon.pack(this.handle, this.packed.world);
    }
    this.paramsKeyPacked = key;
    if (this.overrideColoring) addon.setColoring(this.handle, this.overrideColoring.colorOf);
    this.topologyDirty = false;
  }

  flushTopology(solver) { this.pack(solver); }
  prepareTopologyChange() { this.topologyDirty = true; }

  // step(solver) -> ms spent encoding (backend.js:1393); asynchronous on the device.
  step(solver) {
    if (this.topologyDirty || !this.handle) this.pack(solver);
    // the grab as the WebGPU backend passes it: uniform state of every step
    // (backend.js:1330-1334); the tool moves grab.target in place
    const g = this.grab;
    if (g) addon.setGrab(this.handle, g.body, Float64Array.from(g.local), Float64Array.from(g.target), g.stiffness);
    else if (this._grabbed) addon.setGrab(this.handle, -1);
    this._grabbed = !!g;
    const t0 = performance.now();
    addon.step(this.handle, 1);
    return performance.now() - t0;
  }

  // The launch configuration tuned on the current state (avbd_autotune).
  autotune(trialSteps = 3) { return addon.autotune(this.handle, trialSteps); }

  async idle() { if (this.handle) addon.synchronize(this.handle); }

  async syncToCPU(solver) {
    if (!this.handle || !this.packed) return;
    addon.readState(this.handle, this.packed.world);
    fromSoA(solver, this.packed);
  }

  async readState() {
    addon.readState(this.handle, this.packed.world);
    return { world: this.packed.world, counters: addon.stats(this.handle) };
  }

  async readColoring() { return addon.readColoring(this.handle); }

  // uploadColoring(entries, offsets, counts) (backend.js:1925): colour buckets
  // of body indices; converted to a colour per body.
  uploadColoring(entries, offsets, counts) {
    const colorOf = new Int32Array(this.packed.world.bodies.count).fill(-1);
    for (let c = 0; c < counts.length; c++)
      for (let k = offsets[c]; k < offsets[c] + counts[c]; k++) colorOf[entries[k]] = c;
    this.overrideColoring = { colorOf, numColors: counts.length };
    addon.setColoring(this.handle, colorOf);
  }

  clearColoringOverride() {
    this.overrideColoring = null;
    if (this.handle) addon.setColoring(this.handle, null);
  }

  updateJointAnchor(joint) {
    const i = this.packed.jointIndex.get(joint);
    if (i !== undefined) addon.updateJointAnchor(this.handle, i, Float64Array.from(joint.rA));
  }

  getConstraintGpuState() { return addon.deviceViews(this.handle); }

  setProfiling(on) {
    this._profiling = !!on;
    if (this.handle) addon.setProfiling(this.handle, this._profiling);
  }

  get lastProfile() { return this.handle ? addon.lastProfile(this.handle) : null; }
  get lastStats() { return this.handle ? addon.stats(this.handle) : { gpuReady: false }; }

  destroyBuffers() {
    if (this.handle) addon.destroy(this.handle);
    this.handle = null;
    this.packed = null;
  }
}
