// Generated constraint kernels: run-time compilation (NVRTC, sm_103a) and the per-component
// constraint entry point that launches them.
//
// The reference writes each AIR once, as a FrameworkEval over an EvalAtRow, and evaluates it on
// the domain with SimdDomainEvaluator (crates/prover/src/constraint_framework/simd_domain.rs);
// its expr module records the same AIR as expression trees (constraint_framework/expr/
// evaluator.rs). Here the recorded expressions become CUDA source (stwo_gb300/codegen.py, or any
// caller that emits the same kernel interface), which this file compiles and loads, so that every
// AIR written against the framework runs on the device without a hand-written kernel.
//
// The generated kernel is `extern "C" __global__ void stwo_generated_constraints(stwo::GenArgs)`
// (codegen_rt.cuh). stwo_eval_constraints_codegen does the rest of ComponentProver::
// evaluate_constraint_quotients_on_domain (component.rs:278-416) as stwo_eval_constraints does:
// it reverses the accumulator's slice of random-coefficient powers, computes the bit-reversed
// vanishing inverses and launches the kernel, which adds row_res * denom_inv to the column.
#include "common.cuh"
#include <cstring>
#include "prover.cuh"
#include "codegen_rt.cuh"
#include <nvrtc.h>
#include <memory>
#include <string>
#include <vector>

#include "codegen_headers.inc"  // kFieldCuh, kCodegenRtCuh: the two headers, as text

namespace stwo {

struct CodegenComponent {
  std::string cubin;
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
  uint32_t n_cols = 0, n_params = 0, n_constraints = 0;
  // Launch shape the generated source declares (stwo_generated_layout): threads per block and
  // rows a block covers per iteration of its row loop.
  uint32_t threads = 128, rows_per_block = 128;
  bool fractions = false;  // the module holds stwo_generated_fractions (LogUp interaction trace)
};

static int32_t nvrtc_compile(const char* src, std::string& cubin) {
  nvrtcProgram prog;
  const char* headers[] = {kFieldCuh, kCodegenRtCuh};
  const char* names[] = {"field.cuh", "codegen_rt.cuh"};
  nvrtcResult r = nvrtcCreateProgram(&prog, src, "stwo_generated.cu", 2, headers, names);
  if (r != NVRTC_SUCCESS) {
    set_error("nvrtcCreateProgram: %s", nvrtcGetErrorString(r));
    return STWO_ERR_CUDA;
  }
  // A source that marks itself (a long straight-line body, cut into blocks by the generator) is
  // compiled with the fast-compile pipeline: the default one takes minutes on such a body.
  const bool fast = std::strstr(src, "// stwo-codegen: fast-compile\n") != nullptr;
  const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo", "--Ofast-compile=mid"};
  r = nvrtcCompileProgram(prog, fast ? 4 : 3, opts);
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    if (n) nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    set_error("generated kernel does not compile: %s\n%.4000s", nvrtcGetErrorString(r), log.c_str());
    return STWO_ERR_INVALID_ARG;
  }
  size_t n = 0;
  r = nvrtcGetCUBINSize(prog, &n);
  if (r == NVRTC_SUCCESS) {
    cubin.assign(n, '\0');
    r = nvrtcGetCUBIN(prog, &cubin[0]);
  }
  nvrtcDestroyProgram(&prog);
  if (r != NVRTC_SUCCESS) {
    set_error("nvrtcGetCUBIN: %s", nvrtcGetErrorString(r));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

static int32_t load(CodegenComponent* c) {
  if (c->kernel) return STWO_OK;
  STWO_CHECK_CUDA(cudaLibraryLoadData(&c->lib, c->cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  cudaError_t e = cudaLibraryGetKernel(&c->kernel, c->lib, "stwo_generated_constraints");
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaLibraryGetKernel(&c->kernel, c->lib, "stwo_generated_fractions");
    c->fractions = e == cudaSuccess;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaLibraryUnload(c->lib);
    c->lib = nullptr;
    c->kernel = nullptr;
    set_error("generated module has neither stwo_generated_constraints nor stwo_generated_fractions: %s",
              cudaGetErrorString(e));
    return STWO_ERR_INVALID_ARG;
  }
  void* d_layout = nullptr;
  size_t bytes = 0;
  if (cudaLibraryGetGlobal(&d_layout, &bytes, c->lib, "stwo_generated_layout") == cudaSuccess && bytes == 8) {
    uint32_t layout[2];
    STWO_CHECK_CUDA(cudaMemcpy(layout, d_layout, 8, cudaMemcpyDeviceToHost));
    STWO_REQUIRE(layout[0] >= 32 && layout[0] <= 1024 && layout[0] % 32 == 0 && layout[1] >= 1,
                 "generated module declares an invalid launch shape (%u, %u)", layout[0], layout[1]);
    c->threads = layout[0];
    c->rows_per_block = layout[1];
  } else {
    cudaGetLastError();  // a source without the declaration takes the default shape
  }
  return STWO_OK;
}

}  // namespace stwo

using namespace stwo;

extern "C" {

stwo_status stwo_codegen_compile(const char* kernel_source, uint32_t n_cols, uint32_t n_params,
                                 uint32_t n_constraints, int load_now, stwo_codegen_component* out) {
  STWO_REQUIRE(kernel_source && out, "null argument");
  *out = nullptr;
  std::unique_ptr<CodegenComponent> c(new CodegenComponent());
  c->n_cols = n_cols;
  c->n_params = n_params;
  c->n_constraints = n_constraints;
  int32_t st = nvrtc_compile(kernel_source, c->cubin);
  if (st) return st;
  if (load_now) {
    st = load(c.get());
    if (st) return st;
  }
  *out = reinterpret_cast<stwo_codegen_component>(c.release());
  return STWO_OK;
}

stwo_status stwo_codegen_cubin(stwo_codegen_component comp, void* h_dst, size_t capacity, size_t* h_size) {
  STWO_REQUIRE(comp && h_size, "null argument");
  const std::string& cubin = reinterpret_cast<CodegenComponent*>(comp)->cubin;
  *h_size = cubin.size();
  if (h_dst) {
    STWO_REQUIRE(capacity >= cubin.size(), "capacity %zu below the cubin's %zu bytes", capacity, cubin.size());
    std::memcpy(h_dst, cubin.data(), cubin.size());
  }
  return STWO_OK;
}

stwo_status stwo_codegen_from_cubin(const void* h_cubin, size_t size, uint32_t n_cols, uint32_t n_params,
                                    uint32_t n_constraints, int load_now, stwo_codegen_component* out) {
  STWO_REQUIRE(h_cubin && size && out, "null argument");
  *out = nullptr;
  std::unique_ptr<CodegenComponent> c(new CodegenComponent());
  c->n_cols = n_cols;
  c->n_params = n_params;
  c->n_constraints = n_constraints;
  c->cubin.assign(static_cast<const char*>(h_cubin), size);
  if (load_now) {
    int32_t st = load(c.get());
    if (st) return st;
  }
  *out = reinterpret_cast<stwo_codegen_component>(c.release());
  return STWO_OK;
}

stwo_status stwo_codegen_destroy(stwo_codegen_component comp) {
  auto* c = reinterpret_cast<CodegenComponent*>(comp);
  if (!c) return STWO_OK;
  if (c->lib) cudaLibraryUnload(c->lib);
  delete c;
  return STWO_OK;
}

stwo_status stwo_eval_constraints_codegen(stwo_codegen_component comp, uint32_t trace_log_size,
                                          uint32_t eval_log_size, const uint32_t* const* d_cols, uint32_t n_cols,
                                          const stwo_qm31* h_params, uint32_t n_params,
                                          const stwo_qm31* h_coeff_powers, uint32_t n_coeff_powers,
                                          uint32_t* const d_accum[4], void* stream) {
  auto* c = reinterpret_cast<CodegenComponent*>(comp);
  STWO_REQUIRE(c, "null component");
  STWO_REQUIRE(n_cols == c->n_cols, "the component reads %u columns, %u given", c->n_cols, n_cols);
  STWO_REQUIRE(n_params == c->n_params, "the component names %u parameters, %u given", c->n_params, n_params);
  STWO_REQUIRE(n_coeff_powers == c->n_constraints, "the component has %u constraints, %u coefficient powers given",
               c->n_constraints, n_coeff_powers);
  STWO_REQUIRE(trace_log_size >= 1 && eval_log_size > trace_log_size && eval_log_size <= 28,
               "need 1 <= trace_log_size < eval_log_size <= 28 (got %u, %u)", trace_log_size, eval_log_size);
  STWO_REQUIRE(d_cols || n_cols == 0, "null column table");
  STWO_REQUIRE(n_params == 0 || h_params, "null parameters");
  STWO_REQUIRE(h_coeff_powers || n_coeff_powers == 0, "null coefficient powers");
  STWO_REQUIRE(d_accum && d_accum[0] && d_accum[1] && d_accum[2] && d_accum[3], "null accumulator");
  for (uint32_t i = 0; i < n_cols; i++) STWO_REQUIRE(d_cols[i], "null column %u", i);
  if (c->n_constraints == 0) return STWO_OK;
  int32_t st = load(c);
  if (st) return st;
  STWO_REQUIRE(!c->fractions, "this module is an interaction-trace kernel, not a constraint kernel");

  cudaStream_t s = as_stream(stream);
  const size_t n = c->n_constraints;
  const std::vector<uint32_t> dinv = composition_denom_inv(trace_log_size, eval_log_size);
  // One upload: the column table (2 words per pointer, padded to 16 bytes), the parameters, the
  // powers (the accumulator's slice reversed, component.rs:331; 16-byte aligned for vector loads)
  // and the denominators.
  const size_t w_cols = (2 * (size_t)n_cols + 3) & ~(size_t)3, w_par = 4 * (size_t)n_params, w_pow = 4 * n;
  std::vector<uint32_t> host(w_cols + w_par + w_pow + dinv.size());
  std::memcpy(host.data(), d_cols, n_cols * sizeof(void*));
  for (size_t i = 0; i < n_params; i++)
    for (int j = 0; j < 4; j++) host[w_cols + 4 * i + j] = h_params[i].v[j];
  for (size_t i = 0; i < n; i++)
    for (int j = 0; j < 4; j++) host[w_cols + w_par + 4 * i + j] = h_coeff_powers[n - 1 - i].v[j];
  std::copy(dinv.begin(), dinv.end(), host.begin() + w_cols + w_par + w_pow);
  uint32_t* d = nullptr;
  st = scratch_alloc((void**)&d, host.size() * 4, s);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(d, host.data(), host.size() * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    GenArgs a;
    a.cols = reinterpret_cast<const uint32_t* const*>(d);
    a.params = d + w_cols;
    a.powers = d + w_cols + w_par;
    a.dinv = d + w_cols + w_par + w_pow;
    a.acc0 = d_accum[0];
    a.acc1 = d_accum[1];
    a.acc2 = d_accum[2];
    a.acc3 = d_accum[3];
    a.trace_log = trace_log_size;
    a.eval_log = eval_log_size;
    const uint32_t rows = 1u << eval_log_size;
    const uint32_t threads = c->threads;
    const uint32_t blocks =
        std::min<uint32_t>((rows + c->rows_per_block - 1) / c->rows_per_block, (uint32_t)sm_count() * (2048 / threads));
    void* args[] = {&a};
    e = cudaLaunchKernel((const void*)c->kernel, dim3(blocks), dim3(threads), args, 0, s);
    note_launch();
  }
  scratch_free(d, s);
  if (e != cudaSuccess) {
    set_error("eval_constraints_codegen: %s", cudaGetErrorString(e));
    return STWO_ERR_CUDA;
  }
  return STWO_OK;
}

stwo_status stwo_logup_interaction_codegen(stwo_codegen_component comp, uint32_t log_size,
                                          const uint32_t* const* d_cols, uint32_t n_cols, const stwo_qm31* h_params,
                                          uint32_t n_params, uint32_t* d_out, stwo_qm31* h_claimed_sum,
                                          void* stream) {
  auto* c = reinterpret_cast<CodegenComponent*>(comp);
  STWO_REQUIRE(c && d_out, "null argument");
  STWO_REQUIRE(n_cols == c->n_cols, "the interaction kernel reads %u columns, %u given", c->n_cols, n_cols);
  STWO_REQUIRE(n_params == c->n_params, "the interaction kernel names %u parameters, %u given", c->n_params,
               n_params);
  STWO_REQUIRE(c->n_constraints >= 1, "no LogUp batch");
  STWO_REQUIRE(log_size >= 1 && log_size <= 28, "log_size out of range");
  STWO_REQUIRE(d_cols || n_cols == 0, "null column table");
  STWO_REQUIRE(n_params == 0 || h_params, "null parameters");
  for (uint32_t i = 0; i < n_cols; i++) STWO_REQUIRE(d_cols[i], "null column %u", i);
  int32_t st = load(c);
  if (st) return st;
  STWO_REQUIRE(c->fractions, "this module is a constraint kernel, not an interaction-trace kernel");
  cudaStream_t s = as_stream(stream);
  const size_t w_cols = (2 * (size_t)n_cols + 3) & ~(size_t)3, w_par = 4 * (size_t)n_params;
  std::vector<uint32_t> host(w_cols + w_par + 4);
  std::memcpy(host.data(), d_cols, n_cols * sizeof(void*));
  for (size_t i = 0; i < n_params; i++)
    for (int j = 0; j < 4; j++) host[w_cols + 4 * i + j] = h_params[i].v[j];
  Arena arena(s);
  uint32_t* d = arena.alloc(host.size());
  if (!d) return STWO_ERR_OOM;
  STWO_CHECK_CUDA(cudaMemcpyAsync(d, host.data(), host.size() * 4, cudaMemcpyHostToDevice, s));
  GenArgs a{};
  a.cols = reinterpret_cast<const uint32_t* const*>(d);
  a.params = d + w_cols;
  a.acc0 = d_out;
  a.trace_log = a.eval_log = log_size;
  const uint32_t rows = 1u << log_size;
  const uint32_t blocks =
      std::min<uint32_t>((rows + c->rows_per_block - 1) / c->rows_per_block, (uint32_t)sm_count() * (2048 / c->threads));
  void* args[] = {&a};
  STWO_CHECK_CUDA(cudaLaunchKernel((const void*)c->kernel, dim3(blocks), dim3(c->threads), args, 0, s));
  note_launch();
  // LogupTraceGenerator::finalize_last on the last batch's column (logup.rs:150-190).
  hq claimed;
  st = logup_finalize_last(d_out + (size_t)4 * (c->n_constraints - 1) * rows, log_size, arena, s, &claimed);
  if (st) return st;
  if (h_claimed_sum)
    for (int j = 0; j < 4; j++) h_claimed_sum->v[j] = claimed.v[j];
  return STWO_OK;
}

// A component's constraints at one point, from its recorded expressions compiled to a program
// (stwo_gb300/codegen.py, _point_program): the PointEvaluator of constraint_framework/point.rs,
// on the host. Values 0 .. n_inputs - 1 are the inputs (mask values, parameters, constants); each
// op appends one value:
//   1 add a b | 2 sub a b | 3 mul a b | 4 neg a | 5 inv a | 6 partial a b c d (a + b i + c u + d iu)
//   7 combine n alpha0 z v_0 .. v_{n-1} (sum alpha_{alpha0 + k} v_k - z, the relation entry)
// then n_out and the output value indices; *acc becomes acc * rc + denom_inv * c for each output c
// in order.
stwo_status stwo_point_program_eval(const uint32_t* program, size_t program_len, const stwo_qm31* inputs,
                                    size_t n_inputs, stwo_qm31 rc, stwo_qm31 denom_inv, stwo_qm31* acc) {
  STWO_REQUIRE(program && acc && (inputs || n_inputs == 0), "null argument");
  std::vector<hq> val(n_inputs);
  for (size_t i = 0; i < n_inputs; i++) val[i] = hq_from(inputs[i]);
  size_t pc = 0;
  auto next = [&](uint32_t& w) {
    if (pc >= program_len) return false;
    w = program[pc++];
    return true;
  };
  auto arg = [&](hq& out) {
    uint32_t i;
    if (!next(i) || i >= val.size()) return false;
    out = val[i];
    return true;
  };
  uint32_t n_ops;
  STWO_REQUIRE(next(n_ops), "truncated program");
  val.reserve(n_inputs + n_ops);
  for (uint32_t k = 0; k < n_ops; k++) {
    uint32_t op;
    STWO_REQUIRE(next(op), "truncated program");
    hq a, b, c, d, r;
    switch (op) {
      case 1: case 2: case 3:
        STWO_REQUIRE(arg(a) && arg(b), "bad operand at op %u", k);
        r = op == 1 ? hq_add(a, b) : op == 2 ? hq_sub(a, b) : hq_mul(a, b);
        break;
      case 4: case 5:
        STWO_REQUIRE(arg(a), "bad operand at op %u", k);
        r = op == 4 ? hq_sub(hq_make(0, 0, 0, 0), a) : hq_inv(a);
        break;
      case 6:
        STWO_REQUIRE(arg(a) && arg(b) && arg(c) && arg(d), "bad operand at op %u", k);
        r = hq_add(hq_add(a, hq_mul(b, hq_make(0, 1, 0, 0))),
                   hq_add(hq_mul(c, hq_make(0, 0, 1, 0)), hq_mul(d, hq_make(0, 0, 0, 1))));
        break;
      case 7: {
        uint32_t n, alpha0;
        STWO_REQUIRE(next(n) && next(alpha0) && arg(b) && (size_t)alpha0 + n <= val.size(), "bad combine at op %u", k);
        r = hq_make(0, 0, 0, 0);
        for (uint32_t j = 0; j < n; j++) {
          STWO_REQUIRE(arg(a), "bad combine operand at op %u", k);
          r = hq_add(r, hq_mul(val[alpha0 + j], a));
        }
        r = hq_sub(r, b);
        break;
      }
      default:
        STWO_REQUIRE(false, "unknown op %u at %u", op, k);
    }
    val.push_back(r);
  }
  uint32_t n_out;
  STWO_REQUIRE(next(n_out), "truncated program");
  hq ac = hq_from(*acc), rcq = hq_from(rc), dq = hq_from(denom_inv);
  for (uint32_t k = 0; k < n_out; k++) {
    hq v;
    STWO_REQUIRE(arg(v), "bad output %u", k);
    ac = hq_add(hq_mul(ac, rcq), hq_mul(dq, v));
  }
  for (int i = 0; i < 4; i++) acc->v[i] = ac.v[i];
  return STWO_OK;
}

}  // extern "C"
