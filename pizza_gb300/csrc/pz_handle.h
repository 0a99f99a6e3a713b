// The handle of the C ABI (shared by the host-side translation units).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "pizza_gpu.h"
#include "pz_internal.h"

struct HostInst {
  pz_config c;
  PzInst I;
};

struct PzAdjoint;   // adjoint workspace (pz_adjoint.cu)

struct pz_handle {
  int n_inst = 0;
  std::vector<HostInst> hin;
  std::vector<PzInst> inst;
  double* pool = nullptr;
  long long pool_size = 0;
  PzInst* d_inst = nullptr;
  PzState* d_state = nullptr;
  PzItem* d_ritems = nullptr;
  PzItem* d_mitems = nullptr;
  PzItem* d_order = nullptr;
  int* d_iorder = nullptr;
  PzDev dev{};
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  double* d_rows = nullptr;    // n_inst x PZ_SERIES_COLS gather buffer
  double* d_spec = nullptr;    // 5 x max n_m_max: spectra of one instance
  double* d_spec2d = nullptr;  // 3 x max n_r_max x max n_m_max: (r, m) spectra of one instance
  double* d_bal = nullptr;     // force balances (pz_balance_step, allocated at its first call): the
                               // field block of one instance, 6 complex and 4 real (r, m) planes
  PzItem* d_oitems = nullptr;  // k_obs blocks
  double* d_obs_part = nullptr;
  int* d_obs_cnt = nullptr;
  std::string err = "no error";
  PzAdjoint* adj = nullptr;   // allocated by the first adjoint call
  int adj_grids = 1;           // adjoint sweeps keep the phi-grids of the stage states
  std::vector<PzLaunch> plan;  // kernel launches of one step, in order
  // the plain step with the tensor-core stage: fast instances leave the
  // per-m work lists of fdev and run in k_fast; plan/dev (all instances on
  // the standard kernels) stay for the adjoint sweeps
  std::vector<PzLaunch> fplan;
  PzDev fdev{};
  int n_fast = 0;              // instances on the fast path
  PzItem* d_mitems_std = nullptr;
  int* d_iorder_std = nullptr;
  void* d_fast = nullptr;      // one allocation: fragments, exponents, vectors, descriptors, items
  // lanes of the plain step (every instance on the fast path): the instances
  // split into n_lanes sets, each stepped by its own graph on its own
  // stream, so that one set's phi transforms (FP64-bound) overlap another's
  // tensor-core stage (latency-bound)
  int n_lanes = 1;
  cudaStream_t lane_stream[PZ_LANES_MAX] = {};
  cudaGraphExec_t lane_graph[PZ_LANES_MAX] = {};
  cudaEvent_t lane_fork = nullptr;
  cudaEvent_t lane_join[PZ_LANES_MAX] = {};
  PzDev ldev[PZ_LANES_MAX] = {};
  int* d_lane_inst = nullptr;  // the instances lane by lane (k_cfl's blocks)
};

// host helpers of pz_host.cu
int pz_fail(pz_handle* h, int code, const std::string& msg);
int pz_check_status(pz_handle* h);
void pz_adjoint_free(pz_handle* h);
void pz_adjoint_invalidate(pz_handle* h);   // a stored forward sweep no longer matches the state
