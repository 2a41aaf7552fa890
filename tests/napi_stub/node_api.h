// Declarations of the public Node-API C functions (nodejs.org/api/n-api.html)
// that avbd-sandbox_gb300/napi/avbd_node.cc uses, so that tests can
// compile-check the addon where no Node headers are installed. Not a
// replacement for node_api.h: it only lets the compiler check names, argument
// types and the addon's own C++.
#pragma once
#include <stddef.h>
#include <stdint.h>
typedef struct napi_env__ *napi_env;
typedef struct napi_value__ *napi_value;
typedef struct napi_callback_info__ *napi_callback_info;
typedef enum { napi_ok, napi_invalid_arg, napi_generic_failure } napi_status;
typedef enum { napi_undefined, napi_null, napi_boolean, napi_number, napi_string, napi_symbol, napi_object, napi_function, napi_external, napi_bigint } napi_valuetype;
typedef enum { napi_int8_array, napi_uint8_array, napi_uint8_clamped_array, napi_int16_array, napi_uint16_array, napi_int32_array, napi_uint32_array, napi_float32_array, napi_float64_array, napi_bigint64_array, napi_biguint64_array } napi_typedarray_type;
typedef napi_value (*napi_callback)(napi_env env, napi_callback_info info);
typedef void (*napi_finalize)(napi_env env, void *data, void *hint);
#define NAPI_AUTO_LENGTH SIZE_MAX
#define NODE_GYP_MODULE_NAME avbd_node
#define NAPI_MODULE(name, fn) extern "C" napi_value napi_register_module_v1(napi_env env, napi_value exports) { return fn(env, exports); }
extern "C" {
napi_status napi_throw_error(napi_env, const char *, const char *);
napi_status napi_throw_type_error(napi_env, const char *, const char *);
napi_status napi_get_undefined(napi_env, napi_value *);
napi_status napi_has_named_property(napi_env, napi_value, const char *, bool *);
napi_status napi_get_named_property(napi_env, napi_value, const char *, napi_value *);
napi_status napi_set_named_property(napi_env, napi_value, const char *, napi_value);
napi_status napi_typeof(napi_env, napi_value, napi_valuetype *);
napi_status napi_get_value_bool(napi_env, napi_value, bool *);
napi_status napi_get_value_double(napi_env, napi_value, double *);
napi_status napi_get_value_int32(napi_env, napi_value, int32_t *);
napi_status napi_is_typedarray(napi_env, napi_value, bool *);
napi_status napi_get_typedarray_info(napi_env, napi_value, napi_typedarray_type *, size_t *, void **, napi_value *, size_t *);
napi_status napi_get_cb_info(napi_env, napi_callback_info, size_t *, napi_value *, napi_value *, void **);
napi_status napi_get_value_external(napi_env, napi_value, void **);
napi_status napi_create_external(napi_env, void *, napi_finalize, void *, napi_value *);
napi_status napi_create_object(napi_env, napi_value *);
napi_status napi_create_double(napi_env, double, napi_value *);
napi_status napi_create_int32(napi_env, int32_t, napi_value *);
napi_status napi_create_int64(napi_env, int64_t, napi_value *);
napi_status napi_create_bigint_uint64(napi_env, uint64_t, napi_value *);
napi_status napi_create_arraybuffer(napi_env, size_t, void **, napi_value *);
napi_status napi_create_typedarray(napi_env, napi_typedarray_type, size_t, napi_value, size_t, napi_value *);
napi_status napi_create_function(napi_env, const char *, size_t, napi_callback, void *, napi_value *);
}
