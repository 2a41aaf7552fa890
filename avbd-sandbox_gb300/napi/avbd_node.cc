// avbd_node.cc - Node-API addon over the C ABI of include/avbd_cuda.h, so that
// the sandbox's JavaScript host (src/app/boot.js:2145-2150, where it picks
// `gpuBackend.step(solver)` or `solver.step()`) can drive the CUDA backend as a
// third engine. One JS function per ABI call; scene data crosses as typed
// arrays (no copy on the JS side); every failure throws an Error whose `code`
// is the AVBD_ERR_* status and whose message is avbd_last_error's text.
//
// Build: node-gyp with binding.gyp beside this file, against the in-tree
// libavbd_gb300.so. The JavaScript class mirroring GpuBackend is
// cuda_backend.mjs.
#include <node_api.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/avbd_cuda.h"

namespace {

// The context behind a JS handle; `ctx` is null once destroy() ran, so the
// finaliser does not free it twice.
struct Handle {
  avbd_ctx *ctx = nullptr;
};

napi_value throw_status(napi_env env, const avbd_ctx *ctx, int rc) {
  const std::string code = std::to_string(rc);
  napi_throw_error(env, code.c_str(), avbd_last_error(ctx));
  return nullptr;
}

napi_value undefined(napi_env env) {
  napi_value u;
  napi_get_undefined(env, &u);
  return u;
}

bool has(napi_env env, napi_value obj, const char *name) {
  bool yes = false;
  if (napi_has_named_property(env, obj, name, &yes) != napi_ok || !yes) return false;
  napi_value v;
  napi_valuetype t;
  napi_get_named_property(env, obj, name, &v);
  napi_typeof(env, v, &t);
  return t != napi_undefined && t != napi_null;
}

bool get_number(napi_env env, napi_value obj, const char *name, double *out) {
  if (!has(env, obj, name)) return false;
  napi_value v;
  napi_get_named_property(env, obj, name, &v);
  napi_valuetype t;
  napi_typeof(env, v, &t);
  if (t == napi_boolean) {
    bool b = false;
    napi_get_value_bool(env, v, &b);
    *out = b ? 1.0 : 0.0;
    return true;
  }
  return napi_get_value_double(env, v, out) == napi_ok;
}

// obj[name] as a typed array of `type` holding at least `min_len` elements;
// null when absent (an optional field), and a thrown TypeError when present
// but of the wrong type or too short.
template <class T>
bool get_array(napi_env env, napi_value obj, const char *name, napi_typedarray_type type, size_t min_len, T **out) {
  *out = nullptr;
  if (!has(env, obj, name)) return true;
  napi_value v;
  napi_get_named_property(env, obj, name, &v);
  bool is_ta = false;
  napi_is_typedarray(env, v, &is_ta);
  napi_typedarray_type t;
  size_t len = 0;
  void *data = nullptr;
  if (!is_ta || napi_get_typedarray_info(env, v, &t, &len, &data, nullptr, nullptr) != napi_ok || t != type ||
      len < min_len) {
    const std::string msg = std::string(name) + ": expected a typed array of " + std::to_string(min_len) +
                            (type == napi_float64_array ? " Float64" : type == napi_int32_array ? " Int32" : " Uint32") +
                            " elements";
    napi_throw_type_error(env, nullptr, msg.c_str());
    return false;
  }
  *out = static_cast<T *>(data);
  return true;
}

bool get_object(napi_env env, napi_value obj, const char *name, napi_value *out) {
  if (!has(env, obj, name)) return false;
  napi_get_named_property(env, obj, name, out);
  return true;
}

int32_t get_count(napi_env env, napi_value obj) {
  double c = 0;
  return get_number(env, obj, "count", &c) ? (int32_t)c : 0;
}

// The JS argument list: (handle, ...rest).
struct Args {
  napi_value argv[4];
  size_t argc = 4;
  Handle *h = nullptr;
};

bool args(napi_env env, napi_callback_info info, Args *a, bool need_ctx = true) {
  if (napi_get_cb_info(env, info, &a->argc, a->argv, nullptr, nullptr) != napi_ok) return false;
  if (!need_ctx) return true;
  void *p = nullptr;
  if (a->argc < 1 || napi_get_value_external(env, a->argv[0], &p) != napi_ok || !p) {
    napi_throw_type_error(env, nullptr, "first argument: a CUDA backend handle");
    return false;
  }
  a->h = static_cast<Handle *>(p);
  if (!a->h->ctx) {
    napi_throw_error(env, nullptr, "the CUDA backend handle was destroyed");
    return false;
  }
  return true;
}

}  // namespace

namespace {

// A JS world {bodies, joints, springs, manifolds?, numScenes?, sceneStart?}
// (the field names of cuda_backend.mjs's toSoA) viewed as an avbd_world: the
// pointers alias the typed arrays, valid for the duration of the call.
bool bind_world(napi_env env, napi_value obj, avbd_world *w) {
  std::memset(w, 0, sizeof(*w));
  napi_value b, j, s, m;
  if (get_object(env, obj, "bodies", &b)) {
    avbd_body_soa &B = w->bodies;
    B.count = get_count(env, b);
    const size_t n = (size_t)B.count;
    if (!get_array(env, b, "shape", napi_int32_array, n, &B.shape) ||
        !get_array(env, b, "size", napi_float64_array, 3 * n, &B.size) ||
        !get_array(env, b, "mass", napi_float64_array, n, &B.mass) ||
        !get_array(env, b, "moment", napi_float64_array, 3 * n, &B.moment) ||
        !get_array(env, b, "radius", napi_float64_array, n, &B.radius) ||
        !get_array(env, b, "friction", napi_float64_array, n, &B.friction) ||
        !get_array(env, b, "pos", napi_float64_array, 3 * n, &B.pos) ||
        !get_array(env, b, "quat", napi_float64_array, 4 * n, &B.quat) ||
        !get_array(env, b, "vel", napi_float64_array, 3 * n, &B.vel) ||
        !get_array(env, b, "omega", napi_float64_array, 3 * n, &B.omega) ||
        !get_array(env, b, "prevVel", napi_float64_array, 3 * n, &B.prev_vel) ||
        // contact materials (Rigid.setMaterial, rigid.js:144-214), each optional
        !get_array(env, b, "staticFriction", napi_float64_array, n, &B.static_friction) ||
        !get_array(env, b, "dynamicFriction", napi_float64_array, n, &B.dynamic_friction) ||
        !get_array(env, b, "restitution", napi_float64_array, n, &B.restitution) ||
        !get_array(env, b, "contactOffset", napi_float64_array, n, &B.contact_offset) ||
        !get_array(env, b, "restOffset", napi_float64_array, n, &B.rest_offset))
      return false;
  }
  if (get_object(env, obj, "joints", &j)) {
    avbd_joint_soa &J = w->joints;
    J.count = get_count(env, j);
    const size_t n = (size_t)J.count;
    if (!get_array(env, j, "bodyA", napi_int32_array, n, &J.body_a) ||
        !get_array(env, j, "bodyB", napi_int32_array, n, &J.body_b) ||
        !get_array(env, j, "rA", napi_float64_array, 3 * n, &J.r_a) ||
        !get_array(env, j, "rB", napi_float64_array, 3 * n, &J.r_b) ||
        !get_array(env, j, "stiffnessLin", napi_float64_array, n, &J.stiffness_lin) ||
        !get_array(env, j, "stiffnessAng", napi_float64_array, n, &J.stiffness_ang) ||
        !get_array(env, j, "fracture", napi_float64_array, n, &J.fracture) ||
        !get_array(env, j, "penaltyLin", napi_float64_array, 3 * n, &J.penalty_lin) ||
        !get_array(env, j, "penaltyAng", napi_float64_array, 3 * n, &J.penalty_ang) ||
        !get_array(env, j, "lambdaLin", napi_float64_array, 3 * n, &J.lambda_lin) ||
        !get_array(env, j, "lambdaAng", napi_float64_array, 3 * n, &J.lambda_ang) ||
        !get_array(env, j, "broken", napi_int32_array, n, &J.broken) ||
        !get_array(env, j, "order", napi_int32_array, n, &J.order))
      return false;
  }
  if (get_object(env, obj, "springs", &s)) {
    avbd_spring_soa &S = w->springs;
    S.count = get_count(env, s);
    const size_t n = (size_t)S.count;
    if (!get_array(env, s, "bodyA", napi_int32_array, n, &S.body_a) ||
        !get_array(env, s, "bodyB", napi_int32_array, n, &S.body_b) ||
        !get_array(env, s, "rA", napi_float64_array, 3 * n, &S.r_a) ||
        !get_array(env, s, "rB", napi_float64_array, 3 * n, &S.r_b) ||
        !get_array(env, s, "stiffness", napi_float64_array, n, &S.stiffness) ||
        !get_array(env, s, "rest", napi_float64_array, n, &S.rest) ||
        !get_array(env, s, "tearStrain", napi_float64_array, n, &S.tear_strain) ||
        !get_array(env, s, "penalty", napi_float64_array, n, &S.penalty) ||
        !get_array(env, s, "peakStrain", napi_float64_array, n, &S.peak_strain) ||
        !get_array(env, s, "broken", napi_int32_array, n, &S.broken) ||
        !get_array(env, s, "order", napi_int32_array, n, &S.order))
      return false;
  }
  if (get_object(env, obj, "manifolds", &m)) {  // warm-start contacts in, live ones out
    avbd_manifold_soa &M = w->manifolds;
    double cap = 0;
    M.count = get_count(env, m);
    M.capacity = get_number(env, m, "capacity", &cap) ? (int32_t)cap : M.count;
    const size_t n = (size_t)(M.capacity > M.count ? M.capacity : M.count), K = AVBD_MAX_CONTACTS;
    if (!get_array(env, m, "bodyA", napi_int32_array, n, &M.body_a) ||
        !get_array(env, m, "bodyB", napi_int32_array, n, &M.body_b) ||
        !get_array(env, m, "numContacts", napi_int32_array, n, &M.num_contacts) ||
        !get_array(env, m, "basis", napi_float64_array, 9 * n, &M.basis) ||
        !get_array(env, m, "friction", napi_float64_array, n, &M.friction) ||
        !get_array(env, m, "feature", napi_uint32_array, K * n, &M.feature) ||
        !get_array(env, m, "rA", napi_float64_array, 3 * K * n, &M.r_a) ||
        !get_array(env, m, "rB", napi_float64_array, 3 * K * n, &M.r_b) ||
        !get_array(env, m, "c0", napi_float64_array, 3 * K * n, &M.c0) ||
        !get_array(env, m, "penalty", napi_float64_array, 3 * K * n, &M.penalty) ||
        !get_array(env, m, "lambda", napi_float64_array, 3 * K * n, &M.lambda) ||
        !get_array(env, m, "stick", napi_int32_array, K * n, &M.stick) ||
        !get_array(env, m, "order", napi_int32_array, n, &M.order) ||
        !get_array(env, m, "restitutionBias", napi_float64_array, K * n, &M.restitution_bias))
      return false;
  }
  double ns = 0;
  if (get_number(env, obj, "numScenes", &ns) && ns > 1) {
    w->num_scenes = (int32_t)ns;
    if (!get_array(env, obj, "sceneStart", napi_int32_array, (size_t)ns + 1, &w->scene_start)) return false;
  }
  return true;
}

// Solver params (the names of Solver.defaultParams, src/physics/solver.js:92-236,
// plus this backend's own) over avbd_default_params; absent names keep the default.
void bind_params(napi_env env, napi_value obj, avbd_params *p) {
  avbd_default_params(p);
  double v;
  if (get_number(env, obj, "dt", &v)) p->dt = v;
  if (get_number(env, obj, "gravity", &v)) p->gravity = v;
  if (get_number(env, obj, "iterations", &v)) p->iterations = (int32_t)v;
  if (get_number(env, obj, "postStabilize", &v)) p->post_stabilize = v != 0;
  if (get_number(env, obj, "betaLin", &v)) p->beta_lin = v;
  if (get_number(env, obj, "betaAng", &v)) p->beta_ang = v;
  if (get_number(env, obj, "alpha", &v)) p->alpha = v;
  if (get_number(env, obj, "gamma", &v)) p->gamma = v;
  if (get_number(env, obj, "penaltyMin", &v)) p->penalty_min = v;
  if (get_number(env, obj, "penaltyMax", &v)) p->penalty_max = v;
  if (get_number(env, obj, "collisionMargin", &v)) p->collision_margin = v;
  if (get_number(env, obj, "stickThreshold", &v)) p->stick_threshold = v;
  if (get_number(env, obj, "rotatedInertia", &v)) p->rotated_inertia = v != 0;
  if (get_number(env, obj, "springStiffnessRamp", &v)) p->spring_stiffness_ramp = v != 0;
  if (get_number(env, obj, "springGeometricStiffness", &v)) p->spring_geometric_stiffness = v != 0;
  if (get_number(env, obj, "cachedContactJacobians", &v)) p->cached_contact_jacobians = v != 0;
  if (get_number(env, obj, "waitLimit", &v)) p->wait_limit = (int32_t)v;
  if (get_number(env, obj, "neighborWaitLimit", &v)) p->neighbor_wait_limit = (int32_t)v;
  if (get_number(env, obj, "tailDiv", &v)) p->tail_div = (int32_t)v;
  if (get_number(env, obj, "graph", &v)) p->graph = (int32_t)v;
  if (get_number(env, obj, "fp64RatioThreshold", &v)) p->fp64_ratio_threshold = v;
  if (get_number(env, obj, "lanesPerBody", &v)) p->lanes_per_body = (int32_t)v;
  if (get_number(env, obj, "schedule", &v)) p->schedule = (int32_t)v;
  // the WebGPU engine's contact extensions (solver.js:151-162)
  if (get_number(env, obj, "contactModel", &v)) p->contact_model = (int32_t)v;
  if (get_number(env, obj, "contactOffset", &v)) p->contact_offset = v;
  if (get_number(env, obj, "restOffset", &v)) p->rest_offset = v;
  if (get_number(env, obj, "restitutionThreshold", &v)) p->restitution_threshold = v;
  if (get_number(env, obj, "contactPersistence", &v)) p->contact_persistence = v;
}

napi_value make_double_obj(napi_env env, const char *const *names, const double *vals, int n) {
  napi_value o;
  napi_create_object(env, &o);
  for (int k = 0; k < n; k++) {
    napi_value x;
    napi_create_double(env, vals[k], &x);
    napi_set_named_property(env, o, names[k], x);
  }
  return o;
}

void finalize_handle(napi_env, void *data, void *) {
  Handle *h = static_cast<Handle *>(data);
  if (h->ctx) avbd_destroy(h->ctx);
  delete h;
}

// create(params) -> handle
napi_value Create(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a, false)) return nullptr;
  avbd_params p;
  if (a.argc >= 1) bind_params(env, a.argv[0], &p);
  else avbd_default_params(&p);
  avbd_ctx *ctx = nullptr;
  const int rc = avbd_create(&p, &ctx);
  if (rc) return throw_status(env, nullptr, rc);
  Handle *h = new Handle{ctx};
  napi_value ext;
  if (napi_create_external(env, h, finalize_handle, nullptr, &ext) != napi_ok) {
    avbd_destroy(ctx);
    delete h;
    napi_throw_error(env, nullptr, "napi_create_external failed");
    return nullptr;
  }
  return ext;
}

// destroy(handle): frees the device memory now (the handle is dead afterwards)
napi_value Destroy(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_destroy(a.h->ctx);
  a.h->ctx = nullptr;
  return undefined(env);
}

// pack(handle, world)
napi_value Pack(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_world w;
  if (a.argc < 2 || !bind_world(env, a.argv[1], &w)) return nullptr;
  const int rc = avbd_pack(a.h->ctx, &w);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// repack(handle, world, oldBody, oldJoint, oldSpring) -> carried manifolds:
// the identity-preserving repack; each map an Int32Array (new -> old index,
// -1 new) or undefined
napi_value Repack(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_world w;
  if (a.argc < 2 || !bind_world(env, a.argv[1], &w)) return nullptr;
  napi_value holder;
  napi_create_object(env, &holder);
  const char *names[3] = {"oldBody", "oldJoint", "oldSpring"};
  const size_t counts[3] = {(size_t)w.bodies.count, (size_t)w.joints.count, (size_t)w.springs.count};
  int32_t *maps[3] = {nullptr, nullptr, nullptr};
  for (int k = 0; k < 3; k++) {
    napi_valuetype t = napi_undefined;
    if ((size_t)a.argc > (size_t)(2 + k)) napi_typeof(env, a.argv[2 + k], &t);
    if (t == napi_undefined || t == napi_null) continue;
    napi_set_named_property(env, holder, names[k], a.argv[2 + k]);
    if (!get_array(env, holder, names[k], napi_int32_array, counts[k], &maps[k])) return nullptr;
  }
  int64_t carried = 0;
  const int rc = avbd_repack(a.h->ctx, &w, maps[0], maps[1], maps[2], &carried);
  if (rc) return throw_status(env, a.h->ctx, rc);
  napi_value out;
  napi_create_double(env, (double)carried, &out);
  return out;
}

// writeState(handle, world)
napi_value WriteState(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_world w;
  if (a.argc < 2 || !bind_world(env, a.argv[1], &w)) return nullptr;
  const int rc = avbd_write_state(a.h->ctx, &w);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// readState(handle, world): fills the world's typed arrays (those present);
// returns the number of live manifolds when manifold arrays were given
napi_value ReadState(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_world w;
  if (a.argc < 2 || !bind_world(env, a.argv[1], &w)) return nullptr;
  const int rc = avbd_read_state(a.h->ctx, &w);
  if (rc) return throw_status(env, a.h->ctx, rc);
  napi_value n;
  napi_create_int32(env, w.manifolds.count, &n);
  return n;
}

// step(handle, n): queues n steps (asynchronous)
napi_value Step(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  int32_t n = 1;
  if (a.argc >= 2) napi_get_value_int32(env, a.argv[1], &n);
  const int rc = avbd_step(a.h->ctx, n);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// synchronize(handle): GpuBackend.idle()
napi_value Synchronize(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  const int rc = avbd_synchronize(a.h->ctx);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// readColoring(handle) -> {colorOf: Int32Array, numColors}
napi_value ReadColoring(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_stats st;
  int rc = avbd_read_stats(a.h->ctx, &st);
  if (rc) return throw_status(env, a.h->ctx, rc);
  const size_t n = (size_t)st.bodies;
  napi_value ab, arr, num, out;
  void *data = nullptr;
  napi_create_arraybuffer(env, n * sizeof(int32_t), &data, &ab);
  napi_create_typedarray(env, napi_int32_array, n, ab, 0, &arr);
  int32_t k = 0;
  rc = avbd_read_coloring(a.h->ctx, static_cast<int32_t *>(data), &k);
  if (rc) return throw_status(env, a.h->ctx, rc);
  napi_create_int32(env, k, &num);
  napi_create_object(env, &out);
  napi_set_named_property(env, out, "colorOf", arr);
  napi_set_named_property(env, out, "numColors", num);
  return out;
}

// setColoring(handle, Int32Array | null): uploadColoring / overrideColoring
napi_value SetColoring(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  const int32_t *colors = nullptr;
  if (a.argc >= 2) {
    napi_valuetype t;
    napi_typeof(env, a.argv[1], &t);
    if (t != napi_null && t != napi_undefined) {
      napi_value holder;
      napi_create_object(env, &holder);
      napi_set_named_property(env, holder, "colorOf", a.argv[1]);
      avbd_stats st;
      const int rc = avbd_read_stats(a.h->ctx, &st);
      if (rc) return throw_status(env, a.h->ctx, rc);
      int32_t *p = nullptr;
      if (!get_array(env, holder, "colorOf", napi_int32_array, (size_t)st.bodies, &p)) return nullptr;
      colors = p;
    }
  }
  const int rc = avbd_set_coloring(a.h->ctx, colors);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// updateJointAnchor(handle, joint, Float64Array(3))
napi_value UpdateJointAnchor(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  int32_t joint = -1;
  if (a.argc < 3 || napi_get_value_int32(env, a.argv[1], &joint) != napi_ok) {
    napi_throw_type_error(env, nullptr, "updateJointAnchor(handle, joint, rA)");
    return nullptr;
  }
  napi_value holder;
  napi_create_object(env, &holder);
  napi_set_named_property(env, holder, "rA", a.argv[2]);
  double *r = nullptr;
  if (!get_array(env, holder, "rA", napi_float64_array, 3, &r) || !r) return nullptr;
  const int rc = avbd_update_joint_anchor(a.h->ctx, joint, r);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// setGrab(handle, body, Float64Array(3) local, Float64Array(3) target, stiffness); body -1 releases
napi_value SetGrab(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  int32_t body = -1;
  if (a.argc < 2 || napi_get_value_int32(env, a.argv[1], &body) != napi_ok) {
    napi_throw_type_error(env, nullptr, "setGrab(handle, body, local, target, stiffness)");
    return nullptr;
  }
  if (body < 0) {
    const int rc = avbd_set_grab(a.h->ctx, -1, nullptr, nullptr, 0.0);
    return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
  }
  double k = 0;
  if (a.argc < 5 || napi_get_value_double(env, a.argv[4], &k) != napi_ok) {
    napi_throw_type_error(env, nullptr, "setGrab(handle, body, local, target, stiffness)");
    return nullptr;
  }
  napi_value holder;
  napi_create_object(env, &holder);
  napi_set_named_property(env, holder, "local", a.argv[2]);
  napi_set_named_property(env, holder, "target", a.argv[3]);
  double *local = nullptr, *target = nullptr;
  if (!get_array(env, holder, "local", napi_float64_array, 3, &local) || !local) return nullptr;
  if (!get_array(env, holder, "target", napi_float64_array, 3, &target) || !target) return nullptr;
  const int rc = avbd_set_grab(a.h->ctx, body, local, target, k);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// autotune(handle, trialSteps) -> {schedule, lanesPerBody, tailDiv, blocksPerSm, candidates, defaultMs, bestMs}
napi_value Autotune(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  int32_t steps = 3;
  if (a.argc >= 2) napi_get_value_int32(env, a.argv[1], &steps);
  avbd_tuning t;
  const int rc = avbd_autotune(a.h->ctx, steps, &t);
  if (rc) return throw_status(env, a.h->ctx, rc);
  napi_value o, v;
  napi_create_object(env, &o);
  const struct {
    const char *name;
    double value;
  } fields[] = {{"schedule", (double)t.schedule},      {"lanesPerBody", (double)t.lanes_per_body},
                {"tailDiv", (double)t.tail_div},       {"blocksPerSm", (double)t.blocks_per_sm},
                {"candidates", (double)t.candidates},  {"defaultMs", t.default_ms},
                {"bestMs", t.best_ms}};
  for (const auto &f : fields) {
    napi_create_double(env, f.value, &v);
    napi_set_named_property(env, o, f.name, v);
  }
  return o;
}

// setProfiling(handle, on)
napi_value SetProfiling(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  bool on = false;
  if (a.argc >= 2) napi_get_value_bool(env, a.argv[1], &on);
  const int rc = avbd_set_profiling(a.h->ctx, on ? 1 : 0);
  return rc ? throw_status(env, a.h->ctx, rc) : undefined(env);
}

// lastProfile(handle) -> {broadphaseMs, ..., lanesPerBody}
napi_value LastProfile(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_profile p;
  const int rc = avbd_read_profile(a.h->ctx, &p);
  if (rc) return throw_status(env, a.h->ctx, rc);
  static const char *const names[] = {"broadphaseMs", "narrowphaseMs", "prepareMs", "coloringMs", "solveMs",
                                      "stepMs", "candidatePairs", "manifolds", "contacts", "colors",
                                      "fp64Bodies", "npFace", "npEdge", "npExact", "lanesPerBody"};
  const double vals[] = {p.broadphase_ms, p.narrowphase_ms, p.prepare_ms, p.coloring_ms, p.solve_ms, p.step_ms,
                         (double)p.candidate_pairs, (double)p.manifolds, (double)p.contacts, (double)p.colors,
                         (double)p.fp64_bodies, (double)p.np_face, (double)p.np_edge, (double)p.np_exact,
                         (double)p.lanes_per_body};
  return make_double_obj(env, names, vals, 15);
}

// stats(handle) -> GpuBackend.lastStats-like object
napi_value Stats(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_stats st;
  const int rc = avbd_read_stats(a.h->ctx, &st);
  if (rc) return throw_status(env, a.h->ctx, rc);
  static const char *const names[] = {"bodies", "manifolds", "contacts", "candidatePairs", "jointsBroken",
                                      "springsBroken", "colors", "fp64Bodies", "overflow", "steps",
                                      "maxConstraintError", "maxLambda", "maxPenalty"};
  const double vals[] = {(double)st.bodies, (double)st.manifolds, (double)st.contacts, (double)st.candidate_pairs,
                         (double)st.joints_broken, (double)st.springs_broken, (double)st.colors,
                         (double)st.fp64_bodies, (double)st.overflow, (double)st.steps, st.max_constraint_error,
                         st.max_lambda, st.max_penalty};
  return make_double_obj(env, names, vals, 13);
}

// deviceViews(handle) -> device addresses (BigInt) and counts: getConstraintGpuState()
napi_value DeviceViews(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  avbd_device_views v;
  const int rc = avbd_device_views_get(a.h->ctx, &v);
  if (rc) return throw_status(env, a.h->ctx, rc);
  napi_value o;
  napi_create_object(env, &o);
  auto ptr = [&](const char *name, const void *p) {
    napi_value x;
    napi_create_bigint_uint64(env, (uint64_t)(uintptr_t)p, &x);
    napi_set_named_property(env, o, name, x);
  };
  auto cnt = [&](const char *name, int32_t c) {
    napi_value x;
    napi_create_int32(env, c, &x);
    napi_set_named_property(env, o, name, x);
  };
  ptr("bodyPos", v.body_pos);
  ptr("bodyQuat", v.body_quat);
  cnt("bodyCount", v.body_count);
  ptr("jointState", v.joint_state);
  cnt("jointCount", v.joint_count);
  ptr("springState", v.spring_state);
  cnt("springCount", v.spring_count);
  return o;
}

// kernelLaunches(handle) -> number of device kernels since the last pack
napi_value KernelLaunches(napi_env env, napi_callback_info info) {
  Args a;
  if (!args(env, info, &a)) return nullptr;
  int64_t n = 0;
  const int rc = avbd_kernel_launches(a.h->ctx, &n);
  if (rc) return throw_status(env, a.h->ctx, rc);
  napi_value x;
  napi_create_int64(env, n, &x);
  return x;
}

napi_value Init(napi_env env, napi_value exports) {
  struct {
    const char *name;
    napi_callback fn;
  } const table[] = {{"create", Create},
                     {"destroy", Destroy},
                     {"pack", Pack},
                     {"repack", Repack},
                     {"writeState", WriteState},
                     {"readState", ReadState},
                     {"step", Step},
                     {"synchronize", Synchronize},
                     {"readColoring", ReadColoring},
                     {"setColoring", SetColoring},
                     {"updateJointAnchor", UpdateJointAnchor},
                     {"setGrab", SetGrab},
                     {"autotune", Autotune},
                     {"setProfiling", SetProfiling},
                     {"lastProfile", LastProfile},
                     {"stats", Stats},
                     {"deviceViews", DeviceViews},
                     {"kernelLaunches", KernelLaunches}};
  for (const auto &t : table) {
    napi_value f;
    if (napi_create_function(env, t.name, NAPI_AUTO_LENGTH, t.fn, nullptr, &f) != napi_ok ||
        napi_set_named_property(env, exports, t.name, f) != napi_ok)
      return nullptr;
  }
  return exports;
}

}  // namespace

NAPI_MODULE(NODE_GYP_MODULE_NAME, Init)
