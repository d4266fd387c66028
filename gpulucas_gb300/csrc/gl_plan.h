// gl_plan.h -- the plan object shared by the C ABI translation units (internal).
#pragma once
#include <cstdint>
#include <vector>

#include "gl_internal.h"

using gl::FusedGeom;
using gl::IterArgs;
using gl::PlainGeom;
using gl::ResidentGeom;
using gl::Status;

struct gl_plan {
  int p = 0, N = 0, M = 0, LO = 0, n = 0;
  int mode = GL_MODE_FUSED, device = 0;
  double error_limit = 0.4;
  int check_every = 1000;
  int use_graphs = 1;
  cudaStream_t stream = nullptr;
  FusedGeom fg{};
  PlainGeom pg{};
  IterArgs args{};
  std::vector<void*> allocs;
  Status* h_status = nullptr;  // pinned
  int64_t iters_done = 0;
  double run_maxerr = 0.0;
  bool from_state = false;     // next fused iteration loads (digit, hi)
  bool carry_valid = true;     // device (digit, hi) matches the current products
  cudaGraphExec_t gexec = nullptr;
  int gexec_iters = 0;
  // gl_iterate_host_words / gl_iterate_host, one iteration between pinned host buffers:
  // the whole step (copies in, from-state iteration, dicing stored straight into the
  // mapped output buffers and status) as one graph, kept for one set of buffers
  cudaGraphExec_t hw_exec = nullptr;
  int hw_kind = 0;                  // 1: words step, 2: carry-save pair step
  const void* hw_in[2] = {nullptr, nullptr};
  void* hw_out[2] = {nullptr, nullptr};
  void* hw_out_dev[2] = {nullptr, nullptr};  // device addresses of hw_out's mappings
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t device_bytes = 0;
  bool resident = false;        // short length: whole check intervals in one cluster
  ResidentGeom rg{};
  uint8_t* rscratch = nullptr;  // device scratch of the residue kernels
  int32_t* h_res = nullptr;     // pinned: 64 canonical head digits, scalars, flags
};


// gl_plan_create with an explicit SM count for the layout cost model (1 = a member of
// a batch: minimise total work, the batch spreads units over the device).
int gl_plan_create_ex(int p, int N, const gl_plan_opts* opts, int sms_override, gl_plan** out);
// iterations done outside the plan's own launches (by a batch): bookkeeping only
void gl_plan_note_external_iterations(gl_plan* pl, int64_t iters);
// non-blocking stream; level 0: normal priority, 1: the device's highest, 2: between
cudaError_t gl_make_stream(cudaStream_t* s, int level);
// modelled time of the best fused layout for M complex points on `sms` SMs (layout
// cost model units), +inf if no layout exists
double gl_model_iteration_cost(int M, int sms);
// cost of one column-pass unit and one row-pass unit of a fused plan (FP64 model)
double gl_plan_unit_cost(const gl_plan* pl, bool row);
