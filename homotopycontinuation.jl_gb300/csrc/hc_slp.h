// hc_slp.h — host interface between the C ABI (hc_capi.cu) and the straight-line-program
// compiler (hc_slp.cu): a validated program, its CUDA C source, and the kernels NVRTC built
// from it.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "hc_dev.h"

namespace hcd {

// A straight-line program F: C^n → C^n (ModelKit's InstructionSequence,
// src/model_kit/instruction_sequence.jl:1-27) plus the total-degree start system
// G_i = s_i (x_i^{D_i} - 1) it is tracked from; or, with np > 0 parameters at tape slots
// [poff, poff + np), a program F(x; p) tracked as the parameter homotopy
// H(x, t) = F(x; t p + (1 - t) q) (src/homotopies/parameter_homotopy.jl:3-44).
struct SlpProgram {
  int n = 0;
  std::vector<hc_instruction> instr;
  std::vector<double> consts;  // re, im pairs; tape slots [0, nconst)
  int nconst = 0, voff = 0, tape = 0;
  int np = 0, poff = 0;
  std::vector<int> outputs;
  std::vector<int> degrees;
  std::vector<double> scaling;
};

// Check the program (slot ranges, arities, each slot written before it is read, ops the GPU
// evaluator supports); nparams > 0: parameters at slots [poff, poff + nparams), and degrees /
// scaling are not used (may be null). On failure returns an HC_ERR_* code and a message.
int slp_validate(const hc_slp* F, const int32_t* degrees, const double* scaling, int nparams, int poff,
                 SlpProgram& out, std::string& err);

// CUDA C evaluators of the program (values, values + one tangent per lane, Taylor series of
// orders 1..3) prepended to the tracking kernel's sources. Parameters are read at run time
// (the Launch's slp_pq: p then q), so one compiled module serves every (p, q).
std::string slp_codegen(const SlpProgram& P);

// The tracking kernel compiled with one program's evaluators: track_kernel<false> (FP64) or
// <true> (mixed precision).
struct SlpModule {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
  size_t cubin_bytes = 0;
  double compile_seconds = 0;  // 0 when the cubin came from the cache
  bool from_cache = false;
};
// Compile (or fetch from the in-process or on-disk cache, keyed by a hash of the source and
// the compiler options) and load. Returns HC_OK or an HC_ERR_* code with a message.
int slp_build(const std::string& source, bool mixed, SlpModule& out, std::string& err);

}  // namespace hcd
