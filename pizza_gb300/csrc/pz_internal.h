// Internal data layout shared by the host setup (pz_host.cu) and the
// device kernels (pz_kernels.cu).
//
// Everything of a handle lives in one FP64 device pool.  Offsets are counted
// in doubles; complex arrays occupy two doubles per element and start on an
// even offset (16-byte aligned).
//
// Spectral arrays are stored per m: element (m, r) of an instance's field is
// at complex index m*N + r ("m-major": the N radial values of one azimuthal
// wavenumber are contiguous), which is what the per-m solve kernel streams.
// The per-radius phi-transform kernel gathers the same arrays with a stride
// of N and scatters its outputs back: this is the on-device form of pizza's
// m<->r transposes (src/mpi_transpose.f90:209-318).
//
// Matrices are stored column-major (Fortran order): A(i, j) at i + j*n, so
// that thread i of a matrix-vector product reads consecutive addresses.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define PZ_MAX_RADIX 8
#define PZ_SERIES_CAP 1024
#define PZ_RLOOP_G 4        // radii per block of the stage-level phi-transform kernels
#define PZ_RLOOP_PG 576     // k_rloop: radii per block = clamp(PZ_RLOOP_PG / n_phi_max, 1, 8), so
                            // that every block stages about the same 4*576 complex values
#define PZ_SMEM_MAX (227 * 1024)
#define PZ_OBS_RC 16        // k_obs: radii per block
#define PZ_OBS_NP 10        // k_obs: partial sums per block
#define PZ_LANES_MAX 4      // parallel lanes of the plain step's graph
#define PZ_MAX_STAGES 8     // DIRK stages
#define PZ_BT_LD (PZ_MAX_STAGES + 1)
// DIRK tables at o_bt (unscaled, row-major with leading dimension PZ_BT_LD):
// butcher_imp, butcher_exp, then the assembly rows butcher_ass_imp/exp
#define PZ_BT_IMP 0
#define PZ_BT_EXP (PZ_BT_LD * PZ_BT_LD)
#define PZ_BT_AIMP (2 * PZ_BT_LD * PZ_BT_LD)
#define PZ_BT_AEXP (2 * PZ_BT_LD * PZ_BT_LD + PZ_BT_LD)
#define PZ_BT_SIZE (2 * PZ_BT_LD * PZ_BT_LD + 2 * PZ_BT_LD)

// flag bits of PzInst::flags
enum {
  PZF_DIRECT   = 1,    // smat: coupled (omega, psi) solve per m
  PZF_BUO_IMP  = 2,    // implicit buoyancy (buo_term='IMPLICIT')
  PZF_COR_IMP  = 4,    // implicit Coriolis (direct solve only)
  PZF_EK_PUMP  = 8,    // Ekman pumping
  PZF_NON_ROT  = 16,   // non-rotating
  PZF_IMP_CALC = 32,   // scheme computes the implicit term each step
  PZF_T_IS_OM  = 64,   // TdiffFac == ViscFac (Pr = 1, no hyperdiffusion): the
                       // temperature and vorticity operators of each m /= 0 are
                       // the same matrix; one inverse serves both solves
  PZF_INTEG    = 128,  // Chebyshev integration method (cheb_method='integ'),
                       // tau boundary rows, direct streamfunction solve
  PZF_RERR     = 256,  // l_rerror_fix: round-off threshold in the real
                       // Chebyshev derivative recursions of the m = 0 flow
  PZF_CHEM     = 512,  // composition equation (raxi /= 0): update_xi_coll.f90,
                       // update_xi_integ.f90, ChemFac buoyancy
  PZF_FAST     = 1024, // collocation influence-matrix CNAB2 instance whose stage runs in
                       // k_fast (tensor cores, eigen-basis solves) on the plain step
  PZF_INTEG_DENSE = 2048, // integration method with dense per-m inverses in place of the
                          // bordered banded factors (pz_integ_banded(0))
};

// integration-method operators (N x N, column-major, times rnorm, tau rows
// zero) at o_integ + IM_xxx*N*N, shared by instances of equal N and radratio;
// each is I_k [sum_d P_d(r) f^(d)] on Chebyshev coefficients
enum {
  IM_I2R1 = 0,  // I2 [r f]                        (intcheb2rmult1)
  IM_I2R2,      // I2 [r^2 f]                      (intcheb2rmult2)
  IM_I2,        // I2 [f]
  IM_LT0,       // I2 [r^2 f'' + r f']: intcheb2rmult2lapl(m) = LT0 - m^2 I2
  IM_ULAP,      // I2 [r^2 f'' + r f' - f]         (rmult2 - 3 intcheb1rmult1, m = 0 u_phi)
  IM_I4R3,      // I4 [r^3 f]                      (intcheb4rmult3)
  IM_I4R4,      // I4 [r^4 f]                      (intcheb4rmult4)
  IM_Q0,        // intcheb4rmult4laplrot(m)  = Q0 + m^2 Q1
  IM_Q1,
  IM_S0,        // intcheb4rmult4laplrot2(m) = S0 + m^2 S1 + m^4 S2
  IM_S1,
  IM_S2,
  IM_P0,        // I2 [r^2 omega(psi)] = P0 + m^2 P1 (rotating omega of the integ streamfunction);
  IM_P1,        //   intcheb2rmult2laplrot(m) = -(P0 + m^2 P1), the influence-matrix psi operator
  IM_N0,        // intcheb4rmult4lapl(m)  = N0 + m^2 N1 (non-rotating streamfunction, I4 [r^4 Lap psi])
  IM_N1,
  IM_L0,        // intcheb4rmult4lapl2(m) = L0 + m^2 L1 + m^4 L2 (I4 [r^4 Lap^2 psi])
  IM_L1,
  IM_L2,
  IM_COUNT
};

// radial vectors, each N doubles, at o_rad + RV_xxx*N
enum {
  RV_R = 0, RV_OR1, RV_OR2, RV_BETA, RV_DBETA, RV_EKPUMP, RV_EKP_UP, RV_EKP_US,
  RV_EKP_DUSDP, RV_RGRAV, RV_TCOND, RV_DTCOND, RV_HEIGHT, RV_DELXR2, RV_DELXH2,
  RV_WINT,    // rInt_R(f) = sum_r WINT[r] f[r]       (integration.f90:18-55)
  RV_WSIMP,   // simps(f, theta) = sum_r WSIMP[r] f[r] (integration.f90:104-152)
  RV_BCTOP,   // influence-matrix boundary row at r_cmb (update_psi_coll_dmat.f90:1302-1376)
  RV_BCBOT,   // ... at r_icb
  RV_XICOND,  // conducting composition and its radial derivative (radial.f90:194-195)
  RV_DXICOND,
  RV_COUNT
};

// per-N Chebyshev operator block at o_basis + BM_xxx*N*N (column-major)
enum {
  BM_C = 0,   // costf1: physical <-> Chebyshev (DCT-I, self-inverse), dct_fftw.f90:175-238
  BM_D1C,     // Chebyshev coefficients -> physical d/dr       (get_dr, l_dct_in=.false.)
  BM_D2C,     // Chebyshev coefficients -> physical d2/dr2
  BM_D1P,     // physical -> physical d/dr                     (get_dr, l_dct_in=.true.)
  BM_D2P,     // physical -> physical d2/dr2
  BM_RMAT,    // T_k(x_i)    rMat of chebyshev.f90:281-383 (matrix builders)
  BM_DRMAT,   // T_k'(x_i)   drMat
  BM_D2RMAT,  // T_k''(x_i)  d2rMat
  // parity-compact forms (h = N/2, h2 = (N+1)/2), used by the sym_* products:
  BM_CS,      // C, N x h2: column j < h pairs with s_j = x_j + x_{N-1-j} (even k) or
              // a_j = x_j - x_{N-1-j} (odd k); column h (odd N) is the middle point
  BM_D1CS,    // D1c, 2*h2 x h2: row 2i = even-degree columns of row i, 2i+1 = odd
  BM_D2CS,    // D2c, same layout
  BM_D1PS,    // D1p, 2*h2 x h2: row 2i = (D(i,j)+D(i,N-1-j))/2 (j<h), D(i,h) (odd N);
              //      row 2i+1 = (D(i,j)-D(i,N-1-j))/2 (j<h), 0
  BM_D2PS,    // D2p, same layout
  // transposes, for the discrete adjoint (same parity structure):
  BM_CTS,     // C^T, 2*h2 x h2 (layout of BM_D1CS; mirror row = E - O)
  BM_D1CTS,   // D1c^T, N x h2 (layout of BM_CS; even rows pair with a, odd with s)
  BM_D2CTS,   // D2c^T, N x h2 (layout of BM_CS)
  BM_D1PTS,   // D1p^T, 2*h2 x h2 (layout of BM_D1PS)
  BM_COS,     // C in the layout of BM_D1CS (mirror row = E - O), so that C and D1c
              // share one even/odd split of their input
  BM_COUNT
};

// complex fields per instance, each M*N complex, at o_fld + 2*F_xxx*M*N
enum {
  F_US = 0, F_UP, F_OM, F_PSI, F_TEMP, F_DTEMP, F_DVST, F_DVSOM,
  F_XI, F_DXI, F_DVSXI,     // composition, d xi/dr, r u_s xi (zero without composition)
  F_COUNT
};

struct PzInst {
  int N, M, P, mmax, minc, n_max;
  int scheme, nold, nimp, nexp;
  int flags;
  int nstages;              // 1 for the multistep family
  int dirk;                 // DIRK family (src/dirk_schemes.f90)
  int assembly;             // DIRK scheme with an assembly stage
  int exp_mask, imp_mask;   // bit s-1: l_exp_calc(s), l_imp_calc_rhs(s)
  double dirk_gamma;        // wimp_lin(1)/dt
  int nrad;                 // number of phi-FFT stages
  int radix[PZ_MAX_RADIX];
  double CorFac, BuoFac, TdiffFac, ViscFac, ek, tadvz, alpha;
  double ChemFac, XidiffFac;  // composition (namelists.f90:476-522); 0 without it
  int nhf;                    // history fields: 2 (temperature, psi) or 3 (+ composition)
  double dtMax, dtMin, courfac, dt_fac, rnorm;
  double r_cmb, r_icb;
  double nu_vol_den;        // rInt_R(dtcond^2 height r)
  double nu_int_fac;        // denominator of Nu_int
  double sh_vol_den;        // rInt_R(dxicond^2 height r), denominator of Sh_vol
  long long o_rad;          // RV_COUNT*N
  long long o_basis;        // BM_COUNT*N*N (shared by instances of equal N)
  long long o_tw;           // 4*P: exp(-2 pi i k/P), then exp(+2 pi i k/P); shared by equal P
  long long o_gt;           // M*N*N   temperature operator per m
  long long o_gx;           // M*N*N   composition operator per m (get_xiMat / integ xi lhs)
  long long o_gom;          // M*N*N   vorticity operator per m (influence)
  long long o_guphi;        // N*N     m=0 u_phi operator
  long long o_gpsi;         // M*N*N   K = G_psi P C per m: psi_cheb = -K om_cheb (dt independent)
  long long o_aux;          // 4*M*N: om2, om3, psi2, psi3 (Chebyshev space) ; then 4*M infl
  long long o_gsm;          // DIRECT (smat): 4*M*N*N, per m the first N columns of the
                            // inverse of the coupled 2N x 2N operator, complex, column-major
                            // with leading dimension 2N: (omega, psi)_cheb = G rhs
  long long o_bt;           // DIRK tables, PZ_BT_SIZE doubles
  long long o_gass;         // DIRK assembly: M*N*N, psi_cheb = G_ass rhs (get_assMat, dt independent)
  long long o_fld;          // 2*F_COUNT*M*N
  long long o_hist;         // 2*(nhf*(nold+nimp+nexp))*M*N
  long long o_cfl;          // 2*N: dtr, dth
  long long o_series;       // PZ_SERIES_CAP*16
  long long o_integ;        // integration method: IM_COUNT*N*N (shared by equal N, radratio)
  int im_band[IM_COUNT];    // bandwidth of each IM_ operator (max |i-j| of a nonzero)
  // integration method, bordered banded factors (pz_bord.cuh): half band
  // widths (bkw: of the operator, bkl: of the record) and record strides per
  // m in doubles, of the temperature-like operators (temperature,
  // composition, u_phi, vorticity; 2 tau rows, real) and of the
  // streamfunction operator (influence matrix: 2 tau rows, real; direct
  // solve: 4 tau rows, complex)
  int bkw_t, bkl_t, bkw_p, bkl_p;
  long long bstr_t, bstr_p;
  // direct solve with n_r_max above 97: the coupled build's workspace per m
  // in the pool (o_smat_ws, 0 when it fits shared memory)
  long long o_smat_ws, smat_ws_stride;
  int rg;                   // radii per k_rloop block
  double rerr_thr;          // rerror_fac * epsilon with l_rerror_fix, else 0
};

// bordered banded factors of the integration method (pz_bord.cuh): kl of a
// record (the operator's half band width rounded up to 2, 4 or 8) and the
// record's size in entries (doubles, or double2 for a complex operator) for
// order n with nt tau rows
__host__ __device__ inline int bord_kl(int bw) { return bw <= 2 ? 2 : bw <= 4 ? 4 : 8; }
__host__ __device__ inline long long bord_size(int n, int nt, int kl) {
  const long long nb = n - nt;
  return nb * (3 * kl + 2) + 2LL * nt * nb + (long long)nt * nt + n;
}

struct PzState {
  double time;
  double dt[4];
  double wimp[4], wimp_lin[5], wexp[4];
  int n_step;
  int lMatNext, lMat;
  int bridge;               // start_from_another_scheme active this step
  int l_calc_lin;           // implicit term computed this step
  int b_old, b_impl, b_expl;          // ring base of logical slot 1 (next write)
  int r_old, r_impl, r_expl;          // ring base used by this step's rhs
  int status;               // 0 or a negative PZ_E_* code
  int series_count;
  int ab1;                  // first step of a restart takes AB1 explicit weights (l_AB1)
  double w_lhs;             // implicit weight the current operators were built with
};

// history ring accessors: field f in {0: temperature, 1: psi/omega,
// 2: composition}, kind in {0: old, 1: impl, 2: expl}
__host__ __device__ inline long long pz_hist_off(const PzInst& I, int f, int kind, int phys) {
  long long mn2 = 2LL * I.M * I.N;
  int per = I.nold + I.nimp + I.nexp;
  int base = (kind == 0) ? 0 : (kind == 1 ? I.nold : I.nold + I.nimp);
  return I.o_hist + mn2 * ((long long)f * per + base + phys);
}

struct PzItem { int inst; int idx; };   // (instance, r) or (instance, m index)

#include "pz_fast.h"

// launchers (pz_kernels.cu)
struct PzDev {
  const PzInst* inst;       // device array
  PzState* state;           // device array
  double* pool;
  const PzItem* ritems; int n_ritems;     // (inst, r)
  const PzItem* mitems; int n_mitems;     // (inst, m index)
  const PzItem* oitems; int n_oitems;     // (inst, first radius) of the k_obs blocks, PZ_OBS_RC radii
                                          // each, an instance's blocks consecutive
  double* obs_part;                       // n_oitems x PZ_OBS_NP partial sums of k_obs
  int* obs_cnt;                           // n_inst: k_obs blocks done this launch (reset by the last)
  PzItem* order;                          // n_mitems: k_order's layout of the fused first stage
  const int* iorder;                      // n_iorder: instances in work-list order (their m items are
                                          // contiguous in mitems, m ascending)
  int n_iorder;                           // instances of the per-m work list (mitems)
  int n_inst;
  const int* cfl_inst;      // instances of k_cfl's n_inst blocks (null: the block index)
  int any_chem;             // some instance has composition: the step launches the
                            // kernels' composition instantiations
  int maxN, maxP, maxM;
  int smem_build;           // dynamic shared memory of k_build (bytes)
  int smem_rloop;           // dynamic shared memory of k_rloop (bytes)
  // time-step schedule of the adjoint sweeps (null on the plain step):
  // sched_mode 1 takes dt of step k (0-based n_step) from dt_io[inst*sched_n + k]
  // instead of the Courant estimate, 2 records the chosen dt there; rec (if
  // set) receives the state after the dt/weight update of every step.
  double* dt_io;
  PzState* rec;
  int sched_n, sched_mode;
  // grid snapshots of the adjoint sweeps (null on the plain step): k_rloop of
  // stage s stores the c2r grids of a collocation instance's state, rows
  // [r][us + i up, om + i T][P], at slot gsnap_slot0 + s - 1 of
  // gsnap + o_gsnap[inst] (N * 2P values per slot)
  double2* gsnap;
  const long long* o_gsnap;
  int gsnap_slot0;
  // tensor-core stage of the plain step (n_items 0: none)
  PzFastDev fast;
  int fast_maxN;            // largest n_r_max of the fast classes
};

// `only` selects one instance (>= 0) or all of them (-1).
cudaError_t pz_launch_build_static(const PzDev& d, cudaStream_t s);
cudaError_t pz_launch_init_state(const PzDev& d, int only, cudaStream_t s);
cudaError_t pz_launch_start(const PzDev& d, int only, cudaStream_t s);
// kernel kinds of a step; a step launches, for stage s = 1..max_stages,
// k_rloop(s) [k_cfl, k_build after stage 1] k_mloop(s), then k_assemble (if
// any instance has an assembly stage) and k_obs
// (k_order + k_build_mloop replace k_build + k_mloop(1) when every instance is
// a collocation instance with a small build footprint)
enum { PZK_RLOOP = 0, PZK_CFL, PZK_BUILD, PZK_MLOOP, PZK_OBS, PZK_ASSEMBLE, PZK_MLOOP_INTEG, PZK_ORDER,
       PZK_BUILD_MLOOP, PZK_FAST, PZK_KINDS };
struct PzLaunch { int kind, stage; };
cudaError_t pz_launch_step_kernel(const PzDev& d, int kind, int stage, cudaStream_t s);
const char* pz_step_kernel_name(int kind);
cudaError_t pz_launch_obs(const PzDev& d, int only, cudaStream_t s);
cudaError_t pz_launch_balance(const PzDev& d, int inst, int n_m_max, const double* snap, double* vort, double* vp,
                              cudaStream_t s);
cudaError_t pz_launch_spectra(const PzDev& d, int inst, int n_m_max, double* out, double* out2d, cudaStream_t s);
cudaError_t pz_launch_gather_rows(const PzDev& d, double* out, cudaStream_t s);
cudaError_t pz_setup_kernels();
// k_fast (pz_fast.cu): the tensor-core stage of the fast instances, and its
// dynamic shared memory for G instances per block and grids up to maxN
cudaError_t pz_launch_fast(const PzDev& d, cudaStream_t s);
size_t pz_fast_smem_bytes(int G, int maxN);
long long pz_smat_ws_doubles(int n);
size_t pz_build_smem_bytes(int n, bool direct, bool integ);   // k_build shared memory for one instance
size_t pz_rloop_smem_bytes(int P, int M, int G, int nt);     // k_rloop shared memory, G radii per block,
                                                             // nt transforms per radius (2, or 3 with composition)

// host: the integration-method operators of one (N, radratio), IM_COUNT
// column-major N x N blocks, and their bandwidths (pz_integ_ops.cu)
#include <vector>
void pz_integ_operators(int N, double r_icb, double r_cmb, double rnorm, std::vector<double>& out, int* band);
