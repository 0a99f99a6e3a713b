// Arguments and launcher of the stage-level explicit-terms kernels (pz_stage.cu).
#pragma once
#include <cuda_runtime.h>

#include "pz_internal.h"

struct PzExplArgs {
  const PzInst* inst;      // device pointer to the instance descriptor
  double* pool;            // the handle's pool (operators, radial functions)
  const double2* us;       // (n_m, n_r), n_m fastest, physical space
  const double2* up;
  const double2* om;
  const double2* temp;
  double2* dTdt;           // out: dTdt%expl(:,:,istage)   (n_m, n_r)
  double2* dpsidt;         // out: dpsidt%expl(:,:,istage) (n_m, n_r)
  double* dtr;             // out: radial Courant step per radius
  double* dth;             // out: horizontal Courant step per radius
  double2* s_dVsT;         // scratch: n_m_max * n_r_max complex
  double2* s_dVsOm;        // scratch: n_m_max * n_r_max complex
};

size_t pz_expl_scratch_bytes(int n_r_max, int n_m_max);
cudaError_t pz_launch_explicit_terms(const PzExplArgs& a, int N, int M, int P, cudaStream_t s);

// Arguments of instance `inst` of a handle for the explicit-terms kernels,
// without scratch (the caller sets s_dVsT / s_dVsOm), plus its sizes and
// stream.  Validates the handle, the instance index and the array pointers;
// on error returns a PZ_E_* code and records the message in the handle.
struct pz_handle;
int pz_expl_args(pz_handle* h, int inst, const double* us, const double* up, const double* om,
                 const double* temp, double* dTdt_expl, double* dpsidt_expl, double* dtr, double* dth,
                 PzExplArgs* a, int* N, int* M, int* P, cudaStream_t* s);
int pz_record_error(pz_handle* h, int code, const char* msg);
