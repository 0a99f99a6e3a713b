/*
 * pizza_gpu.h -- C ABI of the GB300 (sm_103a) time step for pizza.
 *
 * The library advances one or many independent annulus instances of pizza's
 * rotating quasi-geostrophic Boussinesq convection problem with the
 * reference's collocation method.  It replaces, for each instance, the stage
 * body of pizza's time_loop (src/step_time.f90:216-368): radial_loop
 * (src/radial_loop.f90:231-394), the m<->r transposes
 * (src/step_time.f90:550-626), finish_explicit_assembly and mloop
 * (src/mloop.f90:36-229), the CFL check (src/courant.f90:78-167) and the
 * IMEX bookkeeping of src/multistep_schemes.f90.
 *
 * Conventions
 *  - FP64 throughout.  Complex arrays are interleaved (re, im) doubles, i.e.
 *    Fortran complex(8) / C double _Complex / torch.complex128.
 *  - Spectral arrays use the reference's m-distributed layout f(n_m, n_r),
 *    n_m fastest (src/fields.f90:42-238): element (n_m, n_r) is at
 *    2*(n_m + n_r*n_m_max).  n_r = 0 is the outer boundary r_cmb.
 *  - Host buffers are owned by the caller and copied; device state belongs to
 *    the library.  All work of one handle is ordered on one CUDA stream.
 *  - Every entry point returns PZ_OK (0) or a negative PZ_E* code; nothing
 *    aborts the process (the reference calls abortRun/MPI_Abort instead,
 *    src/useful.f90:18-44).  pz_last_error() gives the message.
 *  - One host thread per handle.
 */
#ifndef PIZZA_GPU_H
#define PIZZA_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define PZ_OK              0
#define PZ_E_ARG          -1  /* invalid argument or configuration           */
#define PZ_E_CUDA         -2  /* CUDA runtime error                          */
#define PZ_E_SINGULAR     -3  /* zero pivot in a matrix (abortRun 'Singular') */
#define PZ_E_DT_TOO_SMALL -4  /* dt < dtMin (multistep_schemes.f90:335-345)  */
#define PZ_E_NONFINITE    -5  /* NaN/Inf in the state                        */
#define PZ_E_UNSUPPORTED  -6  /* option outside the implemented path         */
#define PZ_E_NOMEM        -7  /* device allocation failed                    */

/* time_scheme values (src/multistep_schemes.f90:35-134) */
#define PZ_CNAB2   0
#define PZ_SBDF2   1
#define PZ_SBDF3   2
#define PZ_SBDF4   3
#define PZ_CNLF    4
#define PZ_MODCNAB 5
#define PZ_TVB33   6
/* DIRK IMEX Runge-Kutta schemes (src/dirk_schemes.f90:35-244); those marked
 * (A) end with an assembly stage (assemble_stage, src/step_time.f90:370-384) */
#define PZ_ARS222    10
#define PZ_ARS232    11   /* (A) */
#define PZ_ARS233    12   /* (A) */
#define PZ_SSP222    13   /* (A) */
#define PZ_LSDIRK222 14   /* (A) */
#define PZ_LZ232     15
#define PZ_CK232     16
#define PZ_ARS443    17
#define PZ_BPR353    18
#define PZ_PC2       19
#define PZ_ARS343    20   /* (A) */
#define PZ_MARS343   21   /* (A) */
#define PZ_SSP322    22   /* (A) */
#define PZ_SSP332    23   /* (A) */
#define PZ_SSP433    24   /* (A) */
#define PZ_DP1_242   25   /* 'DP1-242' */
#define PZ_DP2_242   26   /* 'DP2-242' */
#define PZ_LZ453     27
#define PZ_KC343     28   /* (A) */
#define PZ_KC564     29   /* (A) */
#define PZ_KC785     30   /* (A) */
#define PZ_DBM453    31   /* (A) */

/* matrix_solve values (src/namelists.f90:416-421) */
#define PZ_SOLVE_INFLUENCE 0   /* update_psi_coll_dmat: real om/psi solves + 2x2 influence matrix */
#define PZ_SOLVE_DIRECT    1   /* update_psi_coll_smat: coupled 2N complex solve */

/* cheb_method values (src/namelists.f90:379-384) */
#define PZ_CHEB_COLL  0   /* collocation (update_*_coll)                            */
#define PZ_CHEB_INTEG 1   /* sparse Chebyshev integration with tau rows
                             (update_temp_integ, update_psi_integ_smat)             */

/* time_scale values (src/namelists.f90:472-510) */
#define PZ_TS_VISC 0      /* viscous time unit (default)                            */
#define PZ_TS_ROT  1      /* rotation time unit: CorFac = 2, ViscFac = ek           */

/*
 * One instance's namelist values.  Mirrors pizza's input.nml groups &grid,
 * &control, &phys_param (src/namelists.f90:162-189).  Fields not listed take
 * the reference defaults of src/namelists.f90:530-672 (hdif off, container
 * 'sphere', beta_shift 0, no forcing, temperature only).  pz_config_default()
 * fills every field with those defaults.
 */
typedef struct pz_config {
  int    n_r_max;      /* radial collocation points N                       */
  int    n_cheb_max;   /* Chebyshev truncation (<= n_r_max)                  */
  int    m_max;        /* azimuthal truncation; n_phi_max = 3*m_max/minc     */
  int    minc;         /* azimuthal symmetry (1)                            */
  double ra, ek, pr, radratio;
  double g0, g1, g2;   /* gravity profile rgrav = g0 + g1 r/r_o + g2 r_o^2/r^2 */
  int    ktopt, kbott; /* temperature BCs: 1 = fixed temperature            */
  int    ktopv, kbotv; /* velocity BCs: 1 = stress-free, 2 = rigid           */
  int    l_ek_pump;    /* Ekman pumping                                     */
  int    l_non_rot;    /* non-rotating (ek < 0 also selects it)             */
  int    l_temp_advz;  /* vertical advection of the background temperature  */
  int    time_scheme;  /* PZ_CNAB2 ...                                      */
  int    matrix_solve; /* PZ_SOLVE_INFLUENCE / PZ_SOLVE_DIRECT              */
  int    corio_imp;    /* 1 = 'IMPLICIT' (forced explicit with INFLUENCE)   */
  int    buo_imp;      /* 1 = 'IMPLICIT' (reference default)                */
  double dtMax;        /* maximum and initial time step                     */
  double courfac;      /* >= 1e3 selects the scheme's default CFL factor    */
  double alpha;        /* Crank-Nicolson weight (0.5)                       */
  double dt_fac;       /* CFL hysteresis factor (2)                         */
  int    cheb_method;  /* PZ_CHEB_COLL / PZ_CHEB_INTEG                      */
  int    time_scale;   /* PZ_TS_VISC / PZ_TS_ROT                            */
  int    l_rerror_fix; /* round-off threshold in the real m = 0 Chebyshev
                          derivative recursions (radial_derivatives.f90)   */
  double rerror_fac;   /* threshold = rerror_fac * epsilon (500)            */
  double raxi, sc;     /* composition: raxi /= 0 switches on the xi equation
                          (update_xi_coll.f90, update_xi_integ.f90), sc > 0 */
  int    ktopxi, kbotxi; /* composition BCs: 1 = fixed composition          */
  double xicond_fac;   /* rescaling of the conducting composition (1)       */
} pz_config;

typedef struct pz_handle pz_handle;

/* Fill *cfg with the reference defaults (src/namelists.f90:530-672), with
 * n_cheb_max = n_r_max. */
void pz_config_default(pz_config* cfg);

/* Create a batch of n_instances independent instances (sizes may differ) on
 * the current CUDA device.  Builds the radial grids, Chebyshev operators,
 * phi-FFT plans and the time-independent matrices on the device.
 * Replaces pizza's init sequence (src/pizza.f90:64-199) up to, not including,
 * the start fields. */
int pz_create(const pz_config* cfgs, int n_instances, pz_handle** out);

/* Start fields of one instance (src/init_fields.f90:54-258, no checkpoint):
 * zero histories, time = 0, dt(:) = dtMax, then the given physical-space
 * fields us, up, temp (complex (n_m, n_r) arrays, any may be NULL = zero),
 * from which om, dT/dr and the first implicit state are derived on the
 * device.  temp is the perturbation on top of the conducting profile. */
int pz_set_state(pz_handle* h, int inst, const double* us, const double* up,
                 const double* temp);

/* Same as pz_set_state for all instances at once: each pointer (or NULL)
 * addresses the concatenation of the instances' arrays in instance order. */
int pz_set_state_all(pz_handle* h, const double* us, const double* up,
                     const double* temp);

/* pz_set_state with the composition perturbation xi (on top of the
 * conducting profile; NULL = zero) of an instance with raxi /= 0
 * (init_fields.f90:54-258 with l_chem).  pz_set_state leaves xi zero. */
int pz_set_state_xi(pz_handle* h, int inst, const double* us, const double* up,
                    const double* temp, const double* xi);

/* Composition of one instance (complex (n_m, n_r) arrays, either may be
 * NULL): xi and d xi/dr.  Zero without composition. */
int pz_get_state_xi(pz_handle* h, int inst, double* xi, double* dxi);

/* Advance every instance by n_steps time steps: for each step the stage body
 * of time_loop, with the CFL decision, weight update and matrix rebuild done
 * on the device.  The step is captured once in a CUDA graph and replayed.
 * A handle whose instances all run the tensor-core stage steps them in lanes
 * (PZ_TUNE_LANES), each through its own graph on its own stream; the lanes
 * start after the work already on the handle's stream (pz_stream) and that
 * stream waits for them before anything enqueued after pz_step, so callers
 * order their work on pz_stream exactly as with one graph.
 * Asynchronous: returns after enqueueing; pz_sync() waits and reports
 * device-side errors. */
int pz_step(pz_handle* h, int n_steps);

/* Wait for all enqueued work and check the device status words. */
int pz_sync(pz_handle* h);

/* Copy one instance's physical state back: complex (n_m, n_r) arrays (any
 * pointer may be NULL); time and dt(1) scalars (may be NULL). */
int pz_get_state(pz_handle* h, int inst, double* us, double* up, double* om,
                 double* psi, double* temp, double* dtemp, double* time,
                 double* dt);

/* History slots of the IMEX time arrays (type_tarray, src/time_array.f90:11-71)
 * at a step boundary, in the layout of pz_set_state: field 0 temperature,
 * 1 vorticity (u_phi for m = 0), 2 composition (instances with raxi /= 0);
 * kind 0 old, 1 impl, 2 expl; slot 1-based
 * as in dfdt%old(:,:,slot).  Slot 1 of old/impl is the current state's
 * (recomputed from the fields by pz_set_state); expl slot 1 is formed by the
 * next step.  These carry a multistep run across a checkpoint
 * (src/checkpoints.f90:868-924 writes slots 2..n).  pz_set_history
 * overwrites the slot on the device. */
int pz_get_history(pz_handle* h, int inst, int field, int kind, int slot, double* out);
int pz_set_history(pz_handle* h, int inst, int field, int kind, int slot, const double* in);

/* Time, dt history (nexp values for the multistep family, 1 for DIRK) and
 * step count of one instance.  pz_set_step_state restores them after
 * pz_set_state; n_step >= nold - 1 skips the CNAB2 bridge of the first steps
 * (a restart with a full history), and the operators are rebuilt at the next
 * step.  The latest time-series row is recomputed with the restored time. */
int pz_get_step_state(pz_handle* h, int inst, double* time, double* dt, int* n_step);
int pz_set_step_state(pz_handle* h, int inst, double time, const double* dt, int n_step);

/* Snapshot spectra of one instance's current state, computed on the device
 * (calculate_spectra, src/spectra.f90:104-196): out receives n_m_max rows
 * of 5 doubles, for each m the r-integral (rInt_R) of
 * pi cc2real(f(m, r)) r height(r) for f = us, up, om, temp, and the
 * reference's composition column xi2_m, which spectra.f90:183 fills with the
 * temperature's integral when composition is on (zero without it). */
int pz_get_spectra(pz_handle* h, int inst, double* out);

/* The (r, m) spectra of one instance's current state, computed on the
 * device: the integrands us2R, up2R and enstR of calculate_spectra
 * (src/spectra.f90:134-142), pi cc2real(f(m, r)) r height(r) for f = us, up,
 * om, before the r-integration.  out receives 3 * n_r_max * n_m_max doubles:
 * for each of the three fields an (n_m_max, n_r_max) array with m varying
 * fastest, the layout of 2D_spec_avg.TAG (write_2D_spectra,
 * spectra.f90:371-457), whose time averages the caller accumulates. */
int pz_get_spectra_2d(pz_handle* h, int inst, double* out);

/* One step of every instance of the handle, as pz_step(h, 1) followed by
 * pz_sync, that also returns the force balances of instance inst over that
 * step: the terms vort_balance.f90 and vp_balance.f90 collect when
 * l_vort_balance / l_vphi_balance are set and the next step is a log step
 * (src/step_time.f90:156-157), with the hooks of update_om_coll_dmat
 * (src/update_psi_coll_dmat.f90:154-230, :444-556, :590-682).
 * vort: 6 * n_r_max * n_m_max complex (interleaved doubles), the terms buo,
 *   cor, adv, dwdt, visc, pump, each (n_m_max, n_r_max) with m varying fastest;
 *   as in the reference, dwdt of m /= 0 is the new vorticity in Chebyshev
 *   space minus the old one in physical space, over dt, and visc carries no
 *   ViscFac factor.
 * vp: 4 * n_r_max doubles: rey_stress, dvpdt, visc, pump of u_phi(m = 0).
 * The host accumulates them (vort_balance's calc_avg, vp_balance's
 * write_outputs).  Collocation instances with the influence-matrix solve and
 * a multistep scheme (PZ_E_UNSUPPORTED otherwise).  The first call allocates
 * the handle's balance buffers. */
int pz_balance_step(pz_handle* h, int inst, double* vort, double* vp);

/* l_AB1 of read_checkpoint (src/checkpoints.f90:398-425): when set, the
 * first step after pz_set_step_state(..., n_step = 0) takes first-order
 * explicit weights (src/step_time.f90:309-314).  pizza sets it when a run
 * restarts with another Ekman number or radial method. */
int pz_set_restart_ab1(pz_handle* h, int inst, int l_ab1);

/* Time series of one instance: one row per completed step plus the start row,
 * most recent last, at most *n_rows rows (in: capacity, out: count).
 * Row layout (PZ_SERIES_COLS doubles):
 *   time, us2_2D, up2_2D, up2_axi_2D,                 (e_kin, outputs.f90:677)
 *   us2_3D, up2_3D, uz2_3D, up2_axi_3D,               (e_kin_3D, outputs.f90:686)
 *   NuTop, NuBot, Nu_vol, Nu_int, tTop, tBot, beta_t, (heat, outputs.f90:791)
 *   dt,                                                 (dt(1) of the step)
 *   ShTop, ShBot, Sh_vol, xiTop, xiBot, beta_xi        (composition, outputs.f90:825;
 *                                                        zero without composition) */
#define PZ_SERIES_COLS 22
int pz_get_series(pz_handle* h, int inst, double* rows, int* n_rows);

/* Sizes of one instance: n_r_max, n_m_max, n_phi_max. */
int pz_get_dims(pz_handle* h, int inst, int* n_r_max, int* n_m_max, int* n_phi_max);

/* Number of device kernel launches one time step issues (all instances). */
int pz_launches_per_step(pz_handle* h);

/* Latest time-series row of every instance: n_instances x PZ_SERIES_COLS
 * doubles, one device-to-host copy. */
int pz_latest_rows(pz_handle* h, double* rows);

/* The CUDA stream (cudaStream_t) all work of the handle is ordered on, for
 * callers that time with CUDA events or order their own work after it. */
void* pz_stream(pz_handle* h);

/* Run n_steps steps launching the kernels one by one (no graph), with CUDA
 * events between them on the handle's stream; kernel_ms[k] receives the mean
 * device time per step of kernel kind k (k < PZ_KERNEL_KINDS, summed over the
 * stages of a DIRK step), names in pz_kernel_name(k).  Synchronises. */
#define PZ_KERNEL_KINDS 10
int pz_step_profile(pz_handle* h, int n_steps, double* kernel_ms);
const char* pz_kernel_name(int k);

/* Explicit (nonlinear) terms of instance `inst` for one stage, from caller
 * device arrays: replaces transp_Mloc_to_Rloc, radial_loop,
 * transp_Rloc_to_Mloc and finish_explicit_assembly of the collocation
 * influence-matrix path (src/step_time.f90:222-269, src/radial_loop.f90:231-394,
 * src/mloop.f90:169-229).  us, up, om, temp: physical-space complex (n_m, n_r)
 * device arrays (n_m fastest, like the reference's *_Mloc).  Outputs:
 * dTdt_expl and dpsidt_expl, complex (n_m, n_r) device arrays, and dtr, dth,
 * n_r_max doubles each (the per-radius Courant steps of src/courant.f90:41-76,
 * evaluated with the instance's courfac).  Ordered on the handle's stream,
 * asynchronous; device memory for 2*n_m_max*n_r_max complex intermediates is
 * taken with cudaMallocAsync on that stream and released after the call.
 * Collocation instances without composition only (PZ_E_UNSUPPORTED else). */
int pz_explicit_terms(pz_handle* h, int inst, const double* us, const double* up,
                      const double* om, const double* temp, double* dTdt_expl,
                      double* dpsidt_expl, double* dtr, double* dth);

/* No counterpart in the reference.  pz_explicit_terms without any device
 * allocation, for callers that cannot allocate when they need the explicit
 * terms: a host capturing its own CUDA graph, or one whose device memory is all
 * handed out by its own pool allocator.  Same arguments, results and stream
 * as pz_explicit_terms; its intermediates live in a static device array of
 * 2*PZ_NOALLOC_MAX_MN complex values (1 MiB) that every GPU loading the library
 * keeps until the process exits.  Limits and rules:
 *  - n_m_max*n_r_max of the instance must not exceed PZ_NOALLOC_MAX_MN, else
 *    PZ_E_ARG with a message;
 *  - call it with the handle's device current; the first call on a device
 *    looks up the array's device address (cudaGetSymbolAddress), so make that
 *    first call before any stream capture.  The address is kept for the life
 *    of the process: do not call it again on a device after cudaDeviceReset;
 *  - all calls on a device share the array: calls that overlap on the GPU
 *    race, so order them (one stream, or events).  Nothing needs clearing
 *    between calls. */
#define PZ_NOALLOC_MAX_MN 32768
int pz_explicit_terms_noalloc(pz_handle* h, int inst, const double* us, const double* up,
                              const double* om, const double* temp, double* dTdt_expl,
                              double* dpsidt_expl, double* dtr, double* dth);

/* ---- discrete adjoint (the gradient path) ----------------------------------
 * pizza itself has no adjoint; these entry points back the PyTorch
 * autograd.Function of the binding.  The objective of every instance is
 *   J = (1/n_window) * sum over the last n_window states k of
 *       (us2_3D + up2_3D + uz2_3D)(k)          (e_kin_3D, outputs.f90:553-570)
 * and the gradient is taken with respect to the initial temperature
 * perturbation (the temp argument of pz_set_state) and Ra, for a fixed
 * time-step sequence.  The collocation step is covered with the
 * influence-matrix solve and any multistep or DIRK scheme, and with pizza's
 * default direct solve (update_om_coll_smat, the coupled
 * vorticity-streamfunction system with implicit Ekman pumping and, with
 * corio_term='IMPLICIT', implicit Coriolis) and any multistep scheme; one
 * scheme for all instances of the handle.
 *
 * The objective is selected per sweep: PZ_OBJ_EKIN3D (above) or
 * PZ_OBJ_NUTOP, the mean of NuTop = 1 + dT/dr(m=0, r_cmb)/dtcond(r_cmb).
 *
 * pz_adjoint_forward: run n_steps steps from the start state set by
 * pz_set_state/pz_set_state_all (every instance must be at step 0), storing a
 * checkpoint every checkpoint_every steps (<= 0: store every step, no
 * recomputation).  dt_sched (n_inst x n_steps, row per instance, or NULL)
 * prescribes dt of every step; NULL lets the Courant controller choose and
 * records its choice.  J (n_inst) receives the objective, dt_used (n_inst x
 * n_steps, or NULL) the sequence used.  No time-series rows are written.
 * Leaves the handle at the final state. */
#define PZ_OBJ_EKIN3D 0   /* us2_3D + up2_3D + uz2_3D                 */
#define PZ_OBJ_NUTOP  1   /* NuTop (outputs.f90:742-746), r(1) = r_cmb */
int pz_adjoint_forward(pz_handle* h, int objective, int n_steps, int n_window, int checkpoint_every,
                       const double* dt_sched, double* J, double* dt_used);

/* pz_adjoint_backward: gradient of the last forward sweep's objective.
 * dJ_dtemp: per instance a complex (n_m, n_r) array (m fastest, the layout of
 * pz_set_state), instances concatenated, with dJ = Re(sum conj(g) dtemp);
 * dJ_dra (n_inst).  Either may be NULL.  Leaves the handle at the final
 * state of the forward sweep.  Any pz_step, pz_set_state* or pz_set_ra call
 * in between discards the stored sweep. */
int pz_adjoint_backward(pz_handle* h, double* dJ_dtemp, double* dJ_dra);

/* pz_adjoint_grid_snapshots: keep (enable != 0, the default) or drop the
 * phi-grids of the stored stage states.  Kept, they cost 32*n_r_max*n_phi_max
 * bytes per stored state and the backward sweep skips their inverse
 * transforms; a sweep whose grid buffer cannot be allocated runs without them.
 * Enabling takes effect at the next pz_adjoint_forward; disabling frees the
 * grids at once.  The gradient is the same either way. */
int pz_adjoint_grid_snapshots(pz_handle* h, int enable);

/* Change Ra of one instance (BuoFac = Ra/Pr); the operators do not depend on
 * it.  Used for finite-difference checks of dJ/dRa. */
int pz_set_ra(pz_handle* h, int inst, double ra);

/* No counterpart in the reference (its stencils are closed-form functions of
 * src/chebsparselib.f90).  One banded operator of the integration method,
 * as pz_create derives it for a grid (host only, no device needed):
 * `which` in 0..PZ_INTEG_OPS-1 selects I2[r f], I2[r^2 f], I2[f],
 * I2[r^2 f'' + r f'], I2[r^2 f'' + r f' - f], I4[r^3 f], I4[r^4 f], then
 * Q0, Q1 (intcheb4rmult4laplrot = Q0 + m^2 Q1), S0, S1, S2
 * (intcheb4rmult4laplrot2 = S0 + m^2 S1 + m^4 S2), P0, P1
 * (intcheb2rmult2laplrot = -(P0 + m^2 P1)), N0, N1 (intcheb4rmult4lapl
 * = N0 + m^2 N1) and L0, L1, L2 (intcheb4rmult4lapl2 = L0 + m^2 L1 +
 * m^4 L2); all times rnorm with the tau rows zero.  out: n_r_max^2 doubles,
 * column-major; *bandwidth: max |i-j| of a nonzero entry. */
#define PZ_INTEG_OPS 19
int pz_integ_operator(int n_r_max, double radratio, int which, double* out, int* bandwidth);

/* No counterpart in the reference.  Process-wide choice, for handles created
 * afterwards, of the tensor-core stage: with enable = 1 (the default) every
 * instance that runs the collocation step with the influence-matrix solve
 * and CNAB2 (fixed-temperature, no-slip walls, no composition,
 * n_cheb_max = n_r_max <= 97) solves its per-m systems in the eigenbasis of
 * its dt-independent operator, with all operator products on bf16 tensor
 * cores as an exact FP64 emulation; enable = 0 keeps every instance on the
 * dense FP64 kernels.  Both give the reference's step to FP64 rounding.
 * enable < 0 only queries.  Returns the previous setting.  The adjoint
 * entry points always run the dense kernels. */
int pz_fast_path(int enable);

/* Process-wide choice, for handles created afterwards, of how the
 * integration method (cheb_method='integ') solves its per-m tau-bordered
 * systems.  enable = 1: bordered banded LU factors, as the reference's
 * type_bordmat (src/bordered_matrix.f90:137-183 over
 * src/band_matrix.f90:212-261): the banded block is factorised with partial
 * pivoting inside the band when dt changes, the tau rows through a Schur
 * complement, and every stage runs banded sweeps.  enable = 0 (the default,
 * the faster on this GPU): dense per-m inverses applied as dense products
 * with every lane busy.  Both give the reference's step to FP64 rounding.
 * enable < 0 only queries.  Returns the previous setting. */
int pz_integ_banded(int enable);

/* No counterpart in the reference (pizza chooses its MPI transpose variant
 * by timing, src/communications.f90:407-516; this is the same idea for the
 * kernels' launch shapes).  Process-wide tuning table read by pz_create for
 * handles created afterwards:
 *  - PZ_TUNE_FAST_G: instances of one (n_r_max, m) per block of the
 *    tensor-core stage (key ignored; value 1..16, <= 0 restores the default 8);
 *  - PZ_TUNE_RLOOP_RG: radii per block of the phi-transform kernel for
 *    n_phi_max = key (value 1..16 within its shared memory; <= 0 restores the
 *    default clamp(576 / n_phi_max, 1, 8));
 *  - PZ_TUNE_LANES: parallel lanes of a step whose instances all run the
 *    tensor-core stage (key ignored; value 1..4, <= 0 restores the default 2):
 *    the instances are dealt to the lanes in turn and each lane's kernels
 *    run on their own stream inside the step's graph; handles with fewer
 *    than 16 instances per lane take one.
 * pizza_gb300.autotune times the candidates on the device and applies the
 * winners.  PZ_E_ARG for an unknown parameter or a value out of range. */
#define PZ_TUNE_FAST_G   0
#define PZ_TUNE_RLOOP_RG 1
#define PZ_TUNE_LANES    2
int pz_tune_set(int what, int key, int value);

/* No counterpart in the reference.  Eigen-decomposition the tensor-core
 * stage uses for mode m of an n_r_max grid (host only, no device needed):
 * the Laplacian D2 + r^-1 D - m^2 r^-2 on the n = n_r_max - 2 interior
 * collocation points with Dirichlet walls, P = U diag(lam) U^-1.  lam: n
 * doubles, U: n x n row-major (columns of max-norm 1).  PZ_E_SINGULAR when
 * the decomposition fails (then the instance would use the dense kernels). */
int pz_fast_eigen(int n_r_max, double radratio, int m, double* lam, double* U);

/* No counterpart in the reference.  Measured peak issue rates of the current
 * device for the pipes the step runs on, for rooflines: FP64 fused
 * multiply-add (the phi-FFTs and the dense FP64 kernels) and bf16
 * mma.sync m16n8k16 with fp32 accumulation (the tensor-core stage), in
 * TFLOP/s (2 flops per FMA).  Runs two probe kernels of some tens of ms on
 * the default stream; either pointer may be NULL. */
int pz_probe_peaks(double* dfma_tflops, double* mma_bf16_tflops);

/* Release all device memory of the handle. */
int pz_destroy(pz_handle* h);

/* Last error message of the handle (or of the last failed pz_create when h
 * is NULL).  Never NULL. */
const char* pz_last_error(pz_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* PIZZA_GPU_H */
