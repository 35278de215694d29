/*
 * gbk_tools.h — tuning for libgbk: the Kokkos Tools tuning interface
 * implemented as a tool, an in-process tuning table, and the FP32 MLP cost
 * model's training / inference kernels.
 *
 * Kokkos Tools tuning interface: the struct layouts and callback signatures
 * below are those of core/src/impl/Kokkos_Profiling_C_Interface.h:135-227
 * (they are an ABI: a tool must lay them out the same way), and the callback
 * names are the symbols core/src/impl/Kokkos_Profiling.cpp:700-713 resolves
 * with dlsym.  libgbk.so exports them, so KOKKOS_TOOLS_LIBS=libgbk.so makes
 * this library the tuning tool of a Kokkos program: for every tuning context
 * it tries each candidate combination of the declared output variables once
 * (online exhaustive search, timed between begin_context and end_context),
 * then answers with the fastest; a loaded tuning table answers immediately.
 * The built-in tuners it stands beside are core/src/Kokkos_Tuners.hpp:381-746.
 */
#ifndef GBK_TOOLS_H_
#define GBK_TOOLS_H_

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#include "gbk.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Kokkos Tools tuning types (layout of the reference's C interface) ---- */
#define KOKKOS_TOOLS_TUNING_STRING_LENGTH 64
typedef char Kokkos_Tools_Tuning_String[KOKKOS_TOOLS_TUNING_STRING_LENGTH];
union Kokkos_Tools_VariableValue_ValueUnion {
  int64_t int_value;
  double double_value;
  Kokkos_Tools_Tuning_String string_value;
};
union Kokkos_Tools_VariableValue_ValueUnionSet {
  int64_t* int_value;
  double* double_value;
  Kokkos_Tools_Tuning_String* string_value;
};
struct Kokkos_Tools_ValueSet {
  size_t size;
  union Kokkos_Tools_VariableValue_ValueUnionSet values;
};
enum Kokkos_Tools_OptimizationType { Kokkos_Tools_Minimize, Kokkos_Tools_Maximize };
struct Kokkos_Tools_OptimizationGoal {
  size_t type_id;
  enum Kokkos_Tools_OptimizationType goal;
};
struct Kokkos_Tools_ValueRange {
  union Kokkos_Tools_VariableValue_ValueUnion lower;
  union Kokkos_Tools_VariableValue_ValueUnion upper;
  union Kokkos_Tools_VariableValue_ValueUnion step;
  bool openLower;
  bool openUpper;
};
enum Kokkos_Tools_VariableInfo_ValueType { kokkos_value_double, kokkos_value_int64, kokkos_value_string };
enum Kokkos_Tools_VariableInfo_StatisticalCategory {
  kokkos_value_categorical,
  kokkos_value_ordinal,
  kokkos_value_interval,
  kokkos_value_ratio
};
enum Kokkos_Tools_VariableInfo_CandidateValueType { kokkos_value_set, kokkos_value_range, kokkos_value_unbounded };
union Kokkos_Tools_VariableInfo_SetOrRange {
  struct Kokkos_Tools_ValueSet set;
  struct Kokkos_Tools_ValueRange range;
};
struct Kokkos_Tools_VariableInfo {
  enum Kokkos_Tools_VariableInfo_ValueType type;
  enum Kokkos_Tools_VariableInfo_StatisticalCategory category;
  enum Kokkos_Tools_VariableInfo_CandidateValueType valueQuantity;
  union Kokkos_Tools_VariableInfo_SetOrRange candidates;
  void* toolProvidedInfo;
};
struct Kokkos_Tools_VariableValue {
  size_t type_id;
  union Kokkos_Tools_VariableValue_ValueUnion value;
  struct Kokkos_Tools_VariableInfo* metadata;
};

/* ---- the tool's callbacks (symbols looked up by Kokkos) ------------------- */
/* Loading and unloading (core/src/impl/Kokkos_Profiling_C_Interface.h:39-52,
 * typedefs Kokkos_Profiling_initFunction / finalizeFunction).  At finalize,
 * when the environment variable GBK_TOOL_REPORT names a file, the tool writes
 * a summary there: the variables Kokkos declared to it (name, id, value type,
 * candidate count), the number of value requests and contexts, and the best
 * candidate it found for each tuned context. */
struct Kokkos_Profiling_KokkosPDeviceInfo {
  size_t deviceID;
};
void kokkosp_init_library(const int load_seq, const uint64_t interface_version, const uint32_t device_info_count,
                          struct Kokkos_Profiling_KokkosPDeviceInfo* device_info);
void kokkosp_finalize_library(void);
void kokkosp_declare_input_type(const char* name, const size_t id, struct Kokkos_Tools_VariableInfo* info);
void kokkosp_declare_output_type(const char* name, const size_t id, struct Kokkos_Tools_VariableInfo* info);
void kokkosp_request_values(const size_t context_id, const size_t num_context_values,
                            const struct Kokkos_Tools_VariableValue* context_values, const size_t num_tuning_values,
                            struct Kokkos_Tools_VariableValue* tuning_values);
void kokkosp_begin_context(const size_t context_id);
void kokkosp_end_context(const size_t context_id, struct Kokkos_Tools_VariableValue objective);
void kokkosp_declare_optimization_goal(const size_t context_id, const struct Kokkos_Tools_OptimizationGoal goal);

/* Names of the input (context) and output (tuning) variables the GB300 space
 * declares: inputs "gbk.kind" (0 reduce, 1 scan, 2 histogram, 3 segmented),
 * "gbk.op" (reducer code), "gbk.dtype", "gbk.log2n", "gbk.extra"
 * (histogram: log2 bins * 8 + key-entropy bucket; segmented: log2 mean
 * length); outputs "gbk.block", "gbk.items_per_thread", "gbk.ctas_per_sm",
 * "gbk.variant" (fields of gbk_tuning_t). */

/* ---- in-process tuning table ----------------------------------------------- */
/* Entries map (kind, op, dtype, log2n, extra) to a launch configuration.
 * When enabled, every entry point called with tune == NULL looks its call up
 * (nearest log2n of the same kind/op/dtype/extra) and falls back to the
 * library defaults without a match.  Text format, one entry per line:
 *   kind op dtype log2n extra block items_per_thread ctas_per_sm variant */
int gbk_tuner_clear(void);
int gbk_tuner_set(int kind, int op, int dtype, int log2n, int extra, const gbk_tuning_t* cfg);
int gbk_tuner_lookup(int kind, int op, int dtype, int64_t n, int extra, gbk_tuning_t* cfg);
int gbk_tuner_load(const char* path);
int gbk_tuner_save(const char* path);
int gbk_tuner_enable(int on);
int64_t gbk_tuner_size(void);

/* ---- FP32 MLP cost model: 3 layers, H = 64 hidden units, ReLU ------------- */
/* params (device, float): W1[D*64] b1[64] W2[64*64] b2[64] W3[64] b3[1],
 * row-major W[in][out]; gbk_mlp_param_count(D) floats.
 * forward: X[B*D] -> Y[B]; acts (device, >= B*128 floats) keeps the two
 * hidden layers for backward.
 * backward: dY[B] -> grads (same layout as params, overwritten).
 * mse: dY = 2 (Y - T) / B, loss[0] = mean (Y - T)^2.
 * adam: params -= lr * mhat / (sqrt(vhat) + eps), step t >= 1. */
int64_t gbk_mlp_param_count(int D);
int gbk_mlp_forward(const float* X, int64_t B, int D, const float* params, float* acts, float* Y, gbk_stream_t s);
int gbk_mlp_backward(const float* X, int64_t B, int D, const float* params, const float* acts, const float* dY,
                     float* grads, gbk_stream_t s);
int gbk_mlp_mse(const float* Y, const float* T, int64_t B, float* dY, float* loss, gbk_stream_t s);
int gbk_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t P, float lr, float beta1, float beta2,
                 float eps, int t, gbk_stream_t s);

#ifdef __cplusplus
}
#endif
#endif /* GBK_TOOLS_H_ */
