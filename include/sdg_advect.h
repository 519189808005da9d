/*
 * sdg_advect.h -- C ABI of the GB300 (sm_103a) implementation of the SCALE-DG
 * 3D DG advection hot path: upwind face flux, sum-factorised divergence, lift,
 * and the SSP-RK3 stage update.
 *
 * Conventions, identical to the reference's Fortran arrays:
 *   - every array is column-major (first index fastest) and is passed by
 *     address, with no descriptor;
 *   - a field is (Np, NeA) with node n = i + (j-1)*Nq + (k-1)*Nq^2; the
 *     first Np*Ne values are the owned elements, and the halo slots follow;
 *   - VMapM / VMapP / halo_src_map hold 1-BASED flat DOF indices;
 *   - scalars are passed by value (Fortran: bind(C) with the value
 *     attribute);
 *   - `stream` arguments are cudaStream_t passed as void* (NULL means the
 *     legacy default stream).
 *
 * Every entry point returns an int status: SDG_OK (0) on success, a negative
 * SDG_ERR_* code otherwise.  It never aborts the process.  sdg_last_error()
 * returns a message for the calling thread's last failure.  Entry points
 * that take host pointers copy through device memory and synchronise before
 * they return.  Entry points suffixed _dev take device pointers and are
 * asynchronous on `stream`.
 *
 * Threading: there is no mutable global state except the default
 * optimisation type set by sdg_dg_optr_kernel_setup, which mirrors the
 * reference's module variable eval_typeid (mod_dg_optr_kernel.f90:36).
 * A solver handle must be used by one host thread at a time.
 */
#ifndef SDG_ADVECT_H
#define SDG_ADVECT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SDG_OK 0
#define SDG_ERR_INVALID_ARG (-1)   /* bad size, NULL pointer, bad stage ... */
#define SDG_ERR_UNSUPPORTED_ORDER (-2) /* PolyOrder outside 1..15 */
#define SDG_ERR_BAD_OPTTYPE (-3)   /* not "GENERAL" / "OPT1" / "EVENODD", or never set */
#define SDG_ERR_CUDA (-4)          /* a CUDA runtime call failed */
#define SDG_ERR_OUT_OF_MEMORY (-5) /* device or host allocation failed */
#define SDG_ERR_FILE (-6)          /* operator file missing or malformed */
#define SDG_ERR_MESH (-7)          /* index out of range / not the mesh expected */
#define SDG_ERR_TIMEOUT (-8)       /* a bounded wait expired */
#define SDG_ERR_NO_DEVICE (-9)     /* no CUDA device is visible */

/* DGOptrKernel optimisation types (mod_dg_optr_kernel.f90:38-42). */
#define SDG_OPT_GENERAL 1
#define SDG_OPT_OPT1 2
/* The even-odd factorisation of D1D and of the face lift (needs their
 * centro-symmetry, which GLL operators have to rounding): in the solver and
 * batched forms the fused stage with ~30 % fewer FP64 operations in the FP64
 * form and about half the instructions in the FP32 and emulated forms; in
 * cal_tend the even-odd tendency kernel.  Same result to rounding. */
#define SDG_OPT_EVENODD 3

/* Arithmetic of a solver (the reference is FP64 throughout). */
#define SDG_PREC_FP64 0   /* FP64 state and FP64 arithmetic on the DFMA pipe */
#define SDG_PREC_FP32 1   /* FP32 flux/derivative/lift, FP64 RK state */
#define SDG_PREC_FP64_EMU 2 /* FP64 state and RK combine; flux/derivative/lift in
                               double-float (two FP32 numbers, ~48 bits) on the
                               FP32 pipes; <= 1e-12 relative L2 per tendency
                               against FP64 */

const char* sdg_status_string(int status);
const char* sdg_last_error(void);
/* Library version string. */
const char* sdg_version(void);
/* sizeof of a struct of this header by its name ("sdg_server_config",
 * "sdg_request", "sdg_result", "sdg_server_stats"), 0 for another name: lets
 * a binding check its struct layouts against the library's. */
size_t sdg_struct_size(const char* name);
/* Number of visible CUDA devices (0 when none); never fails. */
int sdg_device_count(void);
/* Makes `device` current for the calling host thread (cudaSetDevice). */
int sdg_set_device(int device);
/* Blocks until all work on the current device has finished. */
int sdg_device_synchronize(void);

/* ---- DG operator data -------------------------------------------------- */

/* Reads operator_data/p<p>.dat the way element_init does
 * (mod_mesh.f90:253-263): x1D(Nq), D1D(Nq,Nq), Lift_mat(Nq,Nq,Nq,6), each
 * starting on a new record; D1D_tr = transpose(D1D).  D1D_tr may be NULL. */
int sdg_operator_read(const char* path, int p, double* x1D, double* D1D,
                      double* D1D_tr, double* Lift_mat);

/* Computes the same operators from the mathematics (Gauss-Lobatto-Legendre
 * nodes, Lagrange differentiation matrix, lift = inverse 1-D mass matrix
 * applied to the face node, identity across the face).  No counterpart in the
 * reference, which loads them from files exported by FE-Project; the values
 * agree with operator_data/p*.dat to rounding.  D1D_tr may be NULL. */
int sdg_operator_generate(int p, double* x1D, double* D1D, double* D1D_tr,
                          double* Lift_mat);
/* The FP64 even-odd tables the EVENODD forms build from an order's operators
 * (host computation, no device): for each axis x, y, z, TE values
 * E(i,l) (i,l < H), O(i,l) (i < HR, l < H), D(i,mid) (i < H, odd N only),
 * A(i) (i < HR), B(i) (i < H), with N = Nq, H = N/2, HR = (N+1)/2 and
 * TE = H*H + HR*H + (N odd ? H : 0) + HR + H; `tables` receives 3*TE values,
 * unscaled.  Returns SDG_ERR_INVALID_ARG when D1D is not centro-antisymmetric
 * or Lift_mat not separable and mirrored (to 1e-13 of the largest entry). */
int sdg_evenodd_tables(int Nq, const double* D1D, const double* Lift_mat,
                       double* tables);

/* ---- drop-in for mod_dg_optr_kernel / mod_advect3d_eq ------------------ */

/* dg_optr_kernel_setup (mod_dg_optr_kernel.f90:45-58): "GENERAL" or "OPT1"
 * (trailing blanks ignored, as trim() does), or "EVENODD" (no reference
 * counterpart: cal_tend uses the even-odd line sums; the operator entry
 * points use the GENERAL order).  Unlike the reference, an unknown string
 * returns SDG_ERR_BAD_OPTTYPE and leaves the setting as it was. */
int sdg_dg_optr_kernel_setup(const char* dgoptr_evaltype);
/* The current default type (SDG_OPT_*), or 0 if never set. */
int sdg_dg_optr_kernel_type(void);

/* advect3d_eq_cal_tend (mod_advect3d_eq.f90:41-85), same argument list and
 * meaning, host pointers.  q,u,v,w,dqdt are (Np,NeA) with halos filled by
 * the caller (main.f90:59, :159-162); only dqdt(:,1:Ne) is written.  Uses the
 * type set by sdg_dg_optr_kernel_setup.  Every VMap entry is range-checked
 * on the device; an index outside 1..Np*NeA returns SDG_ERR_MESH. */
int sdg_advect3d_eq_cal_tend(double* dqdt, const double* q, const double* u,
                             const double* v, const double* w,
                             const double* D1D, const double* D1D_tr,
                             const double* Lift_mat, const int* VMapM,
                             const int* VMapP, const double* normal_fn,
                             const double* Escale, const double* Fscale,
                             int Nq, int Np, int NfpTot, int Ne, int NeA);

/* The same on device pointers, asynchronous on `stream`, with the
 * optimisation type explicit.  `flux_scratch` is caller-owned device memory
 * of NfpTot*Ne doubles for the element-boundary flux (the reference's
 * automatic array ebnd_flux, mod_advect3d_eq.f90:66); `err_flag` is a
 * caller-owned device int that the kernels set to 1 when a VMap index is out
 * of range, and with opt = SDG_OPT_EVENODD to 2 when D1D is not
 * centro-antisymmetric, D1D_tr not its transpose or Lift_mat not separable
 * and mirrored (it is not cleared here).  SDG_OPT_EVENODD honours the
 * caller's per-node Escale and face fluxes; the host-pointer form returns
 * SDG_ERR_INVALID_ARG for flag 2. */
int sdg_advect3d_eq_cal_tend_dev(double* dqdt, const double* q,
                                 const double* u, const double* v,
                                 const double* w, const double* D1D,
                                 const double* D1D_tr, const double* Lift_mat,
                                 const int* VMapM, const int* VMapP,
                                 const double* normal_fn,
                                 const double* Escale, const double* Fscale,
                                 int Nq, int Np, int NfpTot, int Ne, int NeA,
                                 int opt, double* flux_scratch, int* err_flag,
                                 void* stream);

/* Allocation-free form of sdg_advect3d_eq_cal_tend_dev; it has no
 * counterpart in the reference.  For callers that cannot allocate device
 * memory when they need the tendency: a host model that pre-reserves its HBM
 * through its own pool, a request loop that cannot afford the device-wide
 * synchronisation of cudaFree, or code that must not fail for lack of memory
 * mid-step.  The flux scratch and the error flag live in a fixed device array
 * inside the library (16 MiB, held by every GPU that loads the library until
 * exit), so a call allocates nothing; a call needing more than 2^21
 * face-flux values (NfpTot*Ne) is rejected with SDG_ERR_INVALID_ARG.  All
 * calls on a device share that array: calls whose work overlaps on the GPU
 * race and must be serialised by the caller.  The first call on a device
 * looks up the array's device address, so make it before any stream
 * capture.  Synchronous: waits for `stream` and returns SDG_ERR_MESH when a
 * VMap entry is out of range. */
int sdg_advect3d_eq_cal_tend_noalloc(double* dqdt, const double* q,
                                     const double* u, const double* v,
                                     const double* w, const double* D1D,
                                     const double* D1D_tr,
                                     const double* Lift_mat, const int* VMapM,
                                     const int* VMapP,
                                     const double* normal_fn,
                                     const double* Escale,
                                     const double* Fscale, int Nq, int Np,
                                     int NfpTot, int Ne, int NeA, int opt,
                                     void* stream);

/* minval / maxval of n device doubles (main.f90:76-79 prints them for
 * q(:,1:Ne)), exact and independent of reduction order; host results.
 * Synchronises `stream`. */
int sdg_minmax_dev(const double* q, long long n, double* qmin, double* qmax,
                   void* stream);

/* mesh_setup (mod_mesh.f90:74-193) on the device for the periodic box
 * [0,Lx]x[0,Ly]x[0,Lz]: fills caller-owned device arrays with the reference's
 * VMapM, VMapP (NfpTot,Ne; 1-based, periodic faces pointing into the halo
 * buffer in the reference's slot order), normal_fn (NfpTot,Ne,3), Escale
 * (Np,Ne,3), Fscale (NfpTot,Ne), pos_en (Np,Ne,3) and halo_src_map
 * (Nfp*Nhalo).  Any output may be NULL; x1D (host, Nq values) is needed only
 * for pos_en.  The values equal a host mesh_setup bit for bit.  Synchronises
 * `stream` before returning. */
int sdg_mesh_setup_dev(int NeX, int NeY, int NeZ, int p, double Lx, double Ly,
                       double Lz, const double* x1D, int* VMapM, int* VMapP,
                       double* normal_fn, double* Escale, double* Fscale,
                       double* pos_en, int* halo_src_map, void* stream);

/* tensorprod_divlike_dirXYZ (mod_dg_optr_kernel.f90:62-136) over nelem
 * consecutive elements (nelem = 1 is the reference call made per element from
 * mod_advect3d_eq.f90:185-188).  Each array holds nelem blocks of Nq^3
 * values.  Host pointers; uses the type set by sdg_dg_optr_kernel_setup. */
int sdg_tensorprod_divlike_dirXYZ(double* vec_out_x, double* vec_out_y,
                                  double* vec_out_z, const double* Mat,
                                  const double* Mat_tr, const double* vec_in_x,
                                  const double* vec_in_y,
                                  const double* vec_in_z, int Nq, int nelem);
int sdg_tensorprod_divlike_dirXYZ_dev(double* vec_out_x, double* vec_out_y,
                                      double* vec_out_z, const double* Mat,
                                      const double* Mat_tr,
                                      const double* vec_in_x,
                                      const double* vec_in_y,
                                      const double* vec_in_z, int Nq,
                                      int nelem, int opt, void* stream);

/* element_operation_kernel_matvec_gradlike_dirXYZ_P* (opt1 erb:166-219) over
 * nelem elements: the x, y and z derivatives of ONE field, vec_out_x =
 * Mat along i, vec_out_y / vec_out_z = Mat_tr along j / k, running sums.
 * The template's z direction starts with vec_in(i,1,k)*Mat_tr(1,j)
 * (erb:209), a typo; this computes the consistent sum_l vec_in(i,j,l) *
 * Mat_tr(l,k). */
int sdg_tensorprod_gradlike_dirXYZ(double* vec_out_x, double* vec_out_y,
                                   double* vec_out_z, const double* Mat,
                                   const double* Mat_tr, const double* vec_in,
                                   int Nq, int nelem);
int sdg_tensorprod_gradlike_dirXYZ_dev(double* vec_out_x, double* vec_out_y,
                                       double* vec_out_z, const double* Mat,
                                       const double* Mat_tr,
                                       const double* vec_in, int Nq, int nelem,
                                       void* stream);

/* element_operation_kernel_matvec_dirX_P* / dirY_P* / dirZ_P* (opt1
 * erb:51-129) over nelem elements, dir = 1, 2, 3: one running-sum
 * contraction along i with Mat_x, or along j / k with the transposed
 * Mat_y_tr / Mat_z_tr, exactly as the templates take them. */
int sdg_element_matvec_dir(int dir, double* vec_out, const double* Mat,
                           const double* vec_in, int Nq, int nelem);
int sdg_element_matvec_dir_dev(int dir, double* vec_out, const double* Mat,
                               const double* vec_in, int Nq, int nelem,
                               void* stream);

/* element_operation_kernel_matvec_divlike_dirXYZ_var5_P* (opt1
 * erb:347-465): the divlike contraction of 5 variables per element, in the
 * OPT1 summation order (three partial sums for p > 7).  Each array holds
 * nelem blocks of (Nq,Nq,Nq,5) values, outputs in the same layout.  The
 * template's y output index, j + (kv-1)*5*Nq (erb:400), runs past
 * vec_out_y for kv > 1; this writes vec_out_y(i,j,k,v) like x and z. */
int sdg_tensorprod_divlike_dirXYZ_var5(double* vec_out_x, double* vec_out_y,
                                       double* vec_out_z, const double* Mat,
                                       const double* Mat_tr,
                                       const double* vec_in_x,
                                       const double* vec_in_y,
                                       const double* vec_in_z, int Nq,
                                       int nelem);
int sdg_tensorprod_divlike_dirXYZ_var5_dev(double* vec_out_x,
                                           double* vec_out_y,
                                           double* vec_out_z, const double* Mat,
                                           const double* Mat_tr,
                                           const double* vec_in_x,
                                           const double* vec_in_y,
                                           const double* vec_in_z, int Nq,
                                           int nelem, void* stream);

/* tensorprod_Lift_hexahedral (mod_dg_optr_kernel.f90:139-190) over nelem
 * elements: vec_in holds nelem blocks of (Nq,Nq,6), vec_out nelem blocks of
 * Nq^3 values. */
int sdg_tensorprod_Lift_hexahedral(double* vec_out, const double* Lift,
                                   const double* vec_in, int Nq, int nelem);
int sdg_tensorprod_Lift_hexahedral_dev(double* vec_out, const double* Lift,
                                       const double* vec_in, int Nq, int nelem,
                                       void* stream);

/* tensorprod_divlike_dirXYZ (mod_dg_optr_kernel.f90:62-136) in FP32
 * arithmetic over nelem elements of FP32 device arrays (D1D as FP32,
 * column-major).  use_tensor_cores = 1 (Nq = 16, p = 15 only): the three
 * directions as dense products on the tensor cores, lines of a direction
 * batched along M (tcgen05.mma kind::tf32, M = 128, N = K = 16, operands
 * split into TF32 pairs, hi*hi + hi*lo + lo*hi, FP32 accumulation); a wait
 * that runs out sets *err_flag to 1.  use_tensor_cores = 0: the same FP32
 * contraction on the CUDA cores (any Nq).  No summation order of the
 * reference: the results are FP32 approximations of its FP64 ones. */
int sdg_tensorprod_divlike_dirXYZ_f32_dev(float* out_x, float* out_y, float* out_z,
                                          const float* D1D, const float* in_x,
                                          const float* in_y, const float* in_z,
                                          int Nq, int nelem, int use_tensor_cores,
                                          int* err_flag, void* stream);

/* update_halo (mod_mesh.f90:209-221) on a device field f(Np*NeA):
 * f(Np*Ne+b) = f(halo_src_map(b)), b = 1..NhaloNode (1-based map).  A map
 * entry outside the owned DOFs 1..Np*Ne (the only targets mesh_setup
 * produces, mod_mesh.f90:184) is skipped rather than followed. */
int sdg_update_halo_dev(double* f, const int* halo_src_map, int Np, int Ne,
                        int NhaloNode, void* stream);

/* RK stage combine of main.f90:68-73 on device arrays over the owned
 * elements: q = rk_a(s)*q0 + rk_b(s)*(q + dt*dqdt), stage s = 1..3, with the
 * SSP-RK3 coefficients of mod_common.f90:27-30. */
int sdg_rk_stage_dev(double* q, const double* q0, const double* dqdt, int Np,
                     int Ne, int stage, double dt, void* stream);

/* The time loop of main.f90:51-80 on the reference's own device arrays:
 * nstep SSP-RK3 steps of q (Np*NeA; the owned part is advanced), each step
 * q0 = q and per stage update_halo(q) (mod_mesh.f90:209-221),
 * advect3d_eq_cal_tend (mod_advect3d_eq.f90:41-85) and the RK update
 * (main.f90:68-73).  Every array has its reference meaning and layout, as in
 * sdg_advect3d_eq_cal_tend_dev, plus halo_src_map (NhaloNode, 1-based) for
 * the halo slots that VMapP points into.
 *   opt SDG_OPT_EVENODD: one fused launch per stage on two scratch state
 *     buffers -- face flux from VMapM / VMapP, normal_fn and Fscale, the
 *     even-odd line sums with the caller's per-node Escale, the lift and the
 *     RK update.  Halo slots are resolved through halo_src_map once per call
 *     instead of being copied every stage; the velocity factors of the face
 *     flux are formed in a step's first stage and reused in its other two.
 *   opt SDG_OPT_OPT1 / SDG_OPT_GENERAL: the reference's sequence and
 *     summation order (q0 copy, halo update, flux, cal_dqdt, RK: 13 launches
 *     a step).
 * scratch: device memory of at least sdg_advect3d_eq_step_scratch_bytes(Nq,
 * Ne) bytes, 256-byte aligned.  Errors found on the device set *err_flag
 * (not cleared here): 1 for a VMapM / VMapP / halo_src_map entry outside the
 * DOFs it may name, 2 for operators without the even-odd symmetries.  On
 * return the halo slots of q hold the final state's halo values.  Runs
 * asynchronously on `stream`. */
size_t sdg_advect3d_eq_step_scratch_bytes(int Nq, int Ne);
int sdg_advect3d_eq_step_dev(double* q, const double* u, const double* v,
                             const double* w, const double* D1D,
                             const double* D1D_tr, const double* Lift_mat,
                             const int* VMapM, const int* VMapP,
                             const double* normal_fn, const double* Escale,
                             const double* Fscale, const int* halo_src_map,
                             int Nq, int Np, int NfpTot, int Ne, int NeA,
                             int NhaloNode, double dt, int nstep, int opt,
                             void* scratch, size_t scratch_bytes,
                             int* err_flag, void* stream);

/* ---- device-resident solver (replaces the time loop of main.f90:51-80) -- */

/* A periodic structured box of NeX x NeY x NeZ hexahedra of order p on
 * [0,Lx]x[0,Ly]x[0,Lz], exactly the mesh mesh_setup builds
 * (mod_mesh.f90:74-193).  Neighbours are computed from the element index,
 * so no VMap/normal/scale arrays and no halo buffer are stored, and the
 * halo update disappears from the loop.  One step is three fused stage
 * kernels (face flux + lift + divergence + RK combine), reading and writing
 * rotating state buffers. */
typedef struct sdg_solver sdg_solver;

/* D1D(Nq,Nq) and Lift_mat(Nq,Nq,Nq,6) as read from operator_data (or from
 * sdg_operator_generate).  opt = SDG_OPT_GENERAL / SDG_OPT_OPT1 selects the
 * summation order of the divergence (they differ only for p > 7);
 * SDG_OPT_EVENODD the even-odd stage (returns SDG_ERR_INVALID_ARG if
 * D1D or Lift_mat lacks the centro-symmetry beyond 1e-13 relative).
 * precision = SDG_PREC_*.  stream may be NULL.
 * With SDG_OPT_EVENODD and SDG_PREC_FP64 or SDG_PREC_FP64_EMU the solver also
 * holds the face-flux velocity factors of one step (16 bytes per face node,
 * 96/Nq bytes per DOF): the first stage of every step forms them from the
 * current velocity and the other two stages read them. */
int sdg_solver_create(sdg_solver** out, int NeX, int NeY, int NeZ, int p,
                      double Lx, double Ly, double Lz, const double* D1D,
                      const double* Lift_mat, int opt, int precision,
                      void* stream);
/* Checks that caller-built mesh arrays (the reference's mesh_setup outputs,
 * same shapes as in sdg_advect3d_eq_cal_tend) describe exactly the box this
 * solver computes; returns SDG_ERR_MESH at the first difference. */
int sdg_solver_check_mesh(const sdg_solver* s, const int* VMapM,
                          const int* VMapP, const double* normal_fn,
                          const double* Escale, const double* Fscale);
/* Copies the owned part (Np*Ne values) of q,u,v,w from host memory. */
int sdg_solver_upload(sdg_solver* s, const double* q, const double* u,
                      const double* v, const double* w);
/* The same from device memory (asynchronous on the solver's stream). */
int sdg_solver_upload_dev(sdg_solver* s, const double* q, const double* u,
                          const double* v, const double* w);
/* Advances nstep SSP-RK3 steps of size dt (asynchronous). */
int sdg_solver_step(sdg_solver* s, double dt, int nstep);
/* sdg_solver_step bracketed by CUDA events on the solver's stream; waits
 * for the end event and returns the elapsed device time in *ms. */
int sdg_solver_step_timed(sdg_solver* s, double dt, int nstep, double* ms);
/* Copies q (owned part, Np*Ne values) to host memory; synchronises. */
int sdg_solver_download(sdg_solver* s, double* q);
/* Host-to-host solves, pipelined: for each request r < count, uploads
 * q_in[r], u[r], v[r], w[r] (host memory, Np*Ne values each), advances nstep
 * steps of size dt from that state and downloads the result into q_out[r].
 * Two device buffer sets and separate upload / compute / download streams let
 * request r+1's upload and request r-1's download overlap request r's kernels
 * (page-locked host memory is needed for the overlap).  The solver's own
 * state is not touched; the extra buffers are allocated on first use.
 * Synchronises before returning. */
int sdg_solver_solve_host_pipelined(sdg_solver* s, int count,
                                    const double* const* q_in,
                                    const double* const* u,
                                    const double* const* v,
                                    const double* const* w,
                                    double* const* q_out, double dt, int nstep);
/* Device pointer of the current state q (Np*Ne doubles). */
const double* sdg_solver_state_dev(const sdg_solver* s);
/* minval / maxval of the current state over owned DOFs (main.f90:76-79),
 * exact.  Synchronises the solver stream. */
int sdg_solver_minmax(sdg_solver* s, double* qmin, double* qmax);
/* The time loop with its diagnostic output (main.f90:51-80): nstep steps;
 * after each step istep (1-based) with istep % output_interval == 0 the
 * min and max of q are written to records[2k], records[2k+1] for the k-th
 * such step (2 * (nstep / output_interval) doubles).  The loop does not wait
 * for the host between steps; synchronises before returning. */
int sdg_solver_run(sdg_solver* s, double dt, int nstep, int output_interval,
                   double* records);
/* Evaluates the tendency of the current state into dqdt (owned part,
 * host memory), the fused-kernel analogue of advect3d_eq_cal_tend. */
int sdg_solver_tendency(sdg_solver* s, double* dqdt);
/* Kernel launches one step issues (for launch accounting). */
int sdg_solver_launches_per_step(const sdg_solver* s);
/* The solver's stream as void*. */
void* sdg_solver_stream(const sdg_solver* s);
int sdg_solver_destroy(sdg_solver* s);

/* ---- z-slab partitions with a face exchange per stage --------------------
 * The halo exchange that update_halo (mod_mesh.f90:209-221) stands in for
 * in the single-process reference, and that MPI carried in SCALE-DG
 * (README.md:17): the box is split along z into nparts slabs of whole
 * element layers, each partition keeps its owned layers plus one ghost
 * layer on each side, and before every RK stage each partition sends the
 * face plane its neighbours read (bottom owned layer, k = 0 nodes, to the
 * partition below; top owned layer, k = Nq-1 nodes, to the one above,
 * periodically) into the receiver's own ghost layer.  The partitions of one
 * handle live on the current GPU and a message is a device-to-device copy;
 * the plan and the packed buffers are those a multi-GPU run would send
 * between ranks.  Results equal sdg_solver's on the whole box bit for bit. */
typedef struct sdg_slabs sdg_slabs;
/* The split: partition k owns layers [z_begin[k], z_begin[k+1]) (nparts+1
 * entries, as even as possible); its lower ghost layer is filled by
 * partition lo_src[k], its upper one by hi_src[k].  1 <= nparts <= NeZ.
 * Host-only arithmetic. */
int sdg_slab_plan(int NeZ, int nparts, int* z_begin, int* lo_src, int* hi_src);
int sdg_slabs_create(sdg_slabs** out, int NeX, int NeY, int NeZ, int p,
                     double Lx, double Ly, double Lz, const double* D1D,
                     const double* Lift_mat, int opt, int precision, int nparts,
                     void* stream);
/* Host arrays of the whole box (Np*Ne each), as sdg_solver_upload. */
int sdg_slabs_upload(sdg_slabs* s, const double* q, const double* u,
                     const double* v, const double* w);
int sdg_slabs_step(sdg_slabs* s, double dt, int nstep);
int sdg_slabs_download(sdg_slabs* s, double* q);
/* Bytes every partition together sends per RK stage. */
long long sdg_slabs_exchange_bytes(const sdg_slabs* s);
int sdg_slabs_destroy(sdg_slabs* s);

/* ---- batched ensembles: one launch per RK stage and order --------------- */

/* Many independent periodic boxes (orders 1..11, any sizes, each with its own
 * dt) advanced together in FP32-compute / FP64-state form.  A step is a CUDA
 * graph of one launch per RK stage and (order, stage body) group (one block
 * per (instance, element block) work item, or persistent blocks that take
 * the items round-robin) and an index advance: 3 x groups + 1 kernels.
 * dims holds NeX,NeY,NeZ per instance; D1D_by_order / Lift_by_order /
 * x1D_by_order are indexed by the order (entries for absent orders may be
 * NULL; x1D_by_order may be NULL when sdg_ensemble_init_blob is not used).
 * There is no reference counterpart: the reference advances one box. */
typedef struct sdg_ensemble sdg_ensemble;
int sdg_ensemble_create(sdg_ensemble** out, int n, const int* dims,
                        const int* orders, const double* dt,
                        const double* const* D1D_by_order,
                        const double* const* Lift_by_order,
                        const double* const* x1D_by_order, void* stream);
/* Owned q,u,v,w of instance i (Np*Ne values each, host memory). */
int sdg_ensemble_upload(sdg_ensemble* e, int i, const double* q,
                        const double* u, const double* v, const double* w);
/* Device-side initial condition of instance i: Gaussian tracer of width
 * sigma around centre[3] (periodic unit box) in the constant velocity[3]. */
int sdg_ensemble_init_blob(sdg_ensemble* e, int i, const double* centre,
                           double sigma, const double* velocity);
/* Autotuner: picks the stage body (unless sdg_ensemble_set_opt fixed it) and
 * the elements per block for every order present and the block size by
 * timing stage launches on this ensemble; leaves the state as is. */
int sdg_ensemble_tune(sdg_ensemble* e);
int sdg_ensemble_set_epb(sdg_ensemble* e, int p, int epb);
/* Stage body of the batched kernels: SDG_OPT_EVENODD (the default) the
 * even-odd body for every order whose operators have the centro-symmetry;
 * SDG_OPT_GENERAL / SDG_OPT_OPT1 the node body with running sums.  The
 * choice holds for every order and the autotuner keeps it afterwards. */
int sdg_ensemble_set_opt(sdg_ensemble* e, int opt);
/* Block size of every order, or of order p alone. */
int sdg_ensemble_set_threads(sdg_ensemble* e, int threads);
int sdg_ensemble_set_order_threads(sdg_ensemble* e, int p, int threads);
/* threads_by_order receives 12 entries (index = order). */
int sdg_ensemble_get_threads(const sdg_ensemble* e, int* threads_by_order);
/* on = 1: the order groups of a step run on parallel graph branches (one
 * stream each, joined before the index advance); on = 0 (the default): one
 * after the other on the ensemble's stream.  Results are the same either
 * way. */
int sdg_ensemble_set_parallel_groups(sdg_ensemble* e, int on);
/* on = 1: every RK stage is ONE persistent launch over the work items of all
 * orders (blocks take items round-robin and switch on the item's order and
 * body), three launches and the index advance a step; on = 0 (the default):
 * one launch per order group and stage, each kernel compiled for its order
 * with its own register budget, which measured faster.  Results are the same
 * bit for bit either way. */
int sdg_ensemble_set_single_launch(sdg_ensemble* e, int on);
/* eo_by_order receives 12 entries (index = order): 1 where the order's
 * instances run the even-odd body, 0 for the node body or an absent order. */
int sdg_ensemble_get_bodies(const sdg_ensemble* e, int* eo_by_order);
/* epb_by_order receives 12 entries (index = order); threads the block size
 * the present orders share (0 when they differ); grid the largest group's
 * grid. */
int sdg_ensemble_get_config(const sdg_ensemble* e, int* epb_by_order,
                            int* threads, int* grid);
int sdg_ensemble_step(sdg_ensemble* e, int nstep);
int sdg_ensemble_step_timed(sdg_ensemble* e, int nstep, double* ms);
int sdg_ensemble_download(sdg_ensemble* e, int i, double* q);
long long sdg_ensemble_total_dofs(const sdg_ensemble* e);
int sdg_ensemble_launches_per_step(const sdg_ensemble* e);
int sdg_ensemble_destroy(sdg_ensemble* e);

/* ---- serving: continuous batching of advection solves ------------------ */

/* A scheduler thread owns the device.  Requests (a periodic box with its own
 * order 1..11, size, dt and step count, and a Gaussian tracer in a constant
 * velocity generated on the device) are admitted while the HBM budget and the
 * slot count allow; every active request advances one SSP-RK3 step per
 * round of batched launches (FP32 compute, FP64 state), so
 * requests that arrive while others run share the GPU from their next step
 * on.  Finished requests release their memory at once.  No reference
 * counterpart: the reference runs one box per process. */
typedef struct sdg_server sdg_server;
typedef struct {
  int device;               /* CUDA device the server runs on */
  size_t hbm_budget_bytes;  /* admission limit for request state (clamped to
                               90% of the device's free memory) */
  int max_active;           /* requests advanced together at most */
  int max_window_steps;     /* steps between admission points (default 8) */
  int threads;              /* block size of the batched kernels for every
                               order (0: the default of each order) */
  int epb_by_order[16];     /* elements per block by order (0: default) */
  int opt;                  /* stage body: 0 = the measured faster body per order
                               (currently even-odd at every order, where the
                               operators allow it); SDG_OPT_EVENODD = even-odd;
                               SDG_OPT_GENERAL / SDG_OPT_OPT1 = node body
                               (running sums) */
  int threads_by_order[16]; /* block size by order (0: `threads`, else the
                               default of the order) */
  int parallel_groups;      /* 0: the order groups of a step run one after the
                               other on one stream; 1: on parallel streams */
} sdg_server_config;
typedef struct {
  int NeX, NeY, NeZ, p, nstep;
  double dt;
  double centre[3];         /* Gaussian tracer centre in [0,1)^3 */
  double sigma;             /* Gaussian width */
  double velocity[3];       /* constant velocity */
} sdg_request;
typedef struct {
  int status;               /* SDG_OK or the error that ended the request */
  double latency_s;         /* finish - submit */
  double queue_s;           /* admit - submit */
  long long dofs;
} sdg_result;
typedef struct {
  long long completed, steps_run, launches;
  double dof_updates;
  size_t bytes_in_use;
  int active, pending;
  double p50_latency_s, p99_latency_s;
  double span_s;            /* first submit to last finish */
  int fatal_status;
} sdg_server_stats;
int sdg_server_create(sdg_server** out, const sdg_server_config* cfg,
                      const double* const* D1D_by_order,
                      const double* const* Lift_by_order,
                      const double* const* x1D_by_order);
/* Thread-safe.  out_state (Np*Ne doubles, may be NULL) receives the final
 * state; it must stay valid until sdg_server_wait returns. */
int sdg_server_submit(sdg_server* s, const sdg_request* r, double* out_state,
                      uint64_t* ticket);
/* Blocks until the request finishes (SDG_ERR_TIMEOUT after timeout_s). */
int sdg_server_wait(sdg_server* s, uint64_t ticket, double timeout_s,
                    sdg_result* res);
int sdg_server_get_stats(sdg_server* s, sdg_server_stats* out);
/* Host-side fault injection for tests of the failure path: the next rebuild
 * of the active set's device tables after a request completes reports
 * SDG_ERR_OUT_OF_MEMORY as a failed allocation would.  The server then
 * finishes every active request with that status, records it as
 * fatal_status and launches nothing more for them.  No device fault is
 * involved.  No reference counterpart. */
int sdg_server_inject_rebuild_failure(sdg_server* s);
int sdg_server_reset_stats(sdg_server* s);
int sdg_server_destroy(sdg_server* s);

/* ---- measurement helpers ----------------------------------------------- */

/* Device memory for callers of the *_dev entry points that have no CUDA
 * runtime of their own (a Fortran or Python host). */
int sdg_dev_alloc(size_t bytes, void** out);
int sdg_dev_free(void* p);
int sdg_memcpy_h2d(void* dst, const void* src, size_t bytes);
int sdg_memcpy_d2h(void* dst, const void* src, size_t bytes);
/* Device-to-device copy queued on `stream` (the q0 = q copy of the time loop,
 * main.f90:54-57, for callers that drive the per-stage entry points). */
int sdg_memcpy_d2d_async(void* dst, const void* src, size_t bytes, void* stream);
int sdg_memset_dev(void* dst, int value, size_t bytes);

/* Page-locked host memory for fast host<->device copies (cudaHostAlloc). */
int sdg_pinned_alloc(size_t bytes, void** out);
int sdg_pinned_free(void* p);

/* Peak-rate microbenchmark on the current device: dependent-chain-free
 * DFMA, FFMA and FP64<->FP32 conversion throughput, in 1e12 operations per
 * second (an FMA counts as 2 flops in the *_tflops results). */
int sdg_microbench_peaks(double* dfma_tflops, double* ffma_tflops,
                         double* cvt_f64_f32_tops, double* cvt_f32_f64_tops);

#ifdef __cplusplus
}
#endif
#endif
