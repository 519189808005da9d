/*
 * sdg_oracle.h -- CPU restatement of the SCALE-DG kernel-extraction hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference arm of
 * bench.py may call it, to compare against.  The GB300 product library never
 * links, loads or calls it.
 *
 * Parity status: the reference is Fortran and no Fortran compiler is
 * available to build it, and the reference ships no golden vectors or tests.
 * The oracle is therefore "parity unpinned" against reference OUTPUTS.  It is
 * pinned by (i) the reference's own operator files (operator_data/p*.dat,
 * parsed by sdgo_read_operator_file and compared with operators regenerated
 * from the GLL mathematics), and (ii) known-answer tests from the mathematics
 * (exact differentiation of polynomials, free-stream preservation, mass
 * conservation, spectral convergence to the exactly translated sine wave).
 *
 * Conventions (same as the reference, mod_mesh.f90:33-54):
 *   - arrays are Fortran column-major, first index fastest;
 *   - node index n = i + (j-1)*Nq + (k-1)*Nq^2 (1-based), here 0-based;
 *   - VMapM / VMapP / halo_src_map hold 1-BASED flat DOF indices exactly as
 *     the reference builds them (mod_mesh.f90:159-184);
 *   - all arithmetic is IEEE binary64; the library is built with
 *     -ffp-contract=off so that no multiply-add is fused (gfortran -O3 on
 *     baseline x86-64 emits no FMA either).
 */
#ifndef SDG_ORACLE_H
#define SDG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* optimisation type ids, mod_dg_optr_kernel.f90:39-42 */
#define SDGO_GENERAL 1
#define SDGO_OPT1 2

/* RK3 SSP coefficients, mod_common.f90:27-30 */
extern const double sdgo_rk_a[3];
extern const double sdgo_rk_b[3];

/* Reads x1D(Nq), D1D(Nq,Nq), Lift_mat(Nq,Nq,Nq,6) the way
 * element_init does with three list-directed reads (mod_mesh.f90:253-261).
 * Returns 0 on success, -1 if the file cannot be opened, -2 if it is short
 * or malformed.  D1D_tr (mod_mesh.f90:263) is filled when non-NULL. */
int sdgo_read_operator_file(const char* path, int p, double* x1D, double* D1D,
                            double* D1D_tr, double* Lift);

/* Fmask(Nfp,6), 1-based node ids, face order -y,+x,+y,-x,-z,+z
 * (mod_mesh.f90:265-324). */
void sdgo_fmask(int p, int* Fmask);

/* Number of halo elements and of halo face nodes (mod_mesh.f90:96-100). */
int sdgo_nhalo(int NeX, int NeY, int NeZ);

/* mesh_setup (mod_mesh.f90:74-193) for the periodic box [0,Lx]x[0,Ly]x[0,Lz].
 * Output arrays are caller-allocated with the reference shapes:
 *   VMapM, VMapP (NfpTot,Ne); normal_fn (NfpTot,Ne,3); Escale (Np,Ne,3);
 *   Fscale (NfpTot,Ne); pos_en (Np,Ne,3); halo_src_map (Nfp*Nhalo).
 * Any output pointer may be NULL to skip it. */
void sdgo_mesh_setup(int NeX, int NeY, int NeZ, int p, double Lx, double Ly,
                     double Lz, const double* x1D, int* VMapM, int* VMapP,
                     double* normal_fn, double* Escale, double* Fscale,
                     double* pos_en, int* halo_src_map);

/* update_halo (mod_mesh.f90:209-221). */
void sdgo_update_halo(double* f, const int* halo_src_map, int Np, int Ne,
                      int NhaloNode);

/* cal_elembnd_flux (mod_advect3d_eq.f90:89-142). */
void sdgo_cal_elembnd_flux(double* flux, const double* q, const double* u,
                           const double* v, const double* w, const int* VMapM,
                           const int* VMapP, const double* normal_fn,
                           const double* Fscale, int Np, int NfpTot, int Ne,
                           int NeA);

/* tensorprod_divlike_dirXYZ for one element (mod_dg_optr_kernel.f90:62-136),
 * GENERAL order (:197-258) or OPT1 order
 * (mod_dg_optr_kernel_opt1.F90.erb:228-344). */
void sdgo_divlike(double* out_x, double* out_y, double* out_z, const double* D,
                  const double* D_tr, const double* in_x, const double* in_y,
                  const double* in_z, int Nq, int opt);

/* gradlike_dirXYZ for one element (mod_dg_optr_kernel_opt1.F90.erb:166-219),
 * with the z direction contracted along k. */
void sdgo_gradlike(double* out_x, double* out_y, double* out_z, const double* D,
                   const double* D_tr, const double* in, int Nq);

/* divlike_dirXYZ_var5 for one element (erb:347-465): 5 variables, OPT1
 * order; arrays are (Nq,Nq,Nq,5). */
void sdgo_divlike_var5(double* out_x, double* out_y, double* out_z, const double* D,
                       const double* D_tr, const double* in_x, const double* in_y,
                       const double* in_z, int Nq);

/* tensorprod_Lift_hexahedral for one element (mod_dg_optr_kernel.f90:139-190,
 * :262-288; erb:134-157 has the same order). */
void sdgo_lift(double* out, const double* Lift, const double* in, int Nq);

/* cal_dqdt (mod_advect3d_eq.f90:146-201). */
void sdgo_cal_dqdt(double* dqdt, const double* q, const double* u,
                   const double* v, const double* w, const double* flux_bnd,
                   const double* D1D, const double* D1D_tr,
                   const double* Lift, const double* Escale, int Nq, int Np,
                   int NfpTot, int Ne, int NeA, int opt);

/* advect3d_eq_cal_tend (mod_advect3d_eq.f90:41-85).  Returns 0, or -3 if the
 * temporary flux array cannot be allocated. */
int sdgo_cal_tend(double* dqdt, const double* q, const double* u,
                  const double* v, const double* w, const double* D1D,
                  const double* D1D_tr, const double* Lift, const int* VMapM,
                  const int* VMapP, const double* normal_fn,
                  const double* Escale, const double* Fscale, int Nq, int Np,
                  int NfpTot, int Ne, int NeA, int opt);

/* One RK stage combine over owned elements (main.f90:68-73). stage is 0-based. */
void sdgo_rk_stage(double* q, const double* q0, const double* dqdt, int Np,
                   int Ne, int stage, double dt);

/* The time loop of main.f90:51-80: per step q0 <- q, then three stages of
 * update_halo(q), cal_tend, RK combine.  q,u,v,w are (Np,NeA) with the halos
 * of u,v,w already filled (main.f90:159-162).  q0 and dqdt are (Np,NeA)
 * work arrays.  When minmax is non-NULL it receives, for every step,
 * min and max of q over owned DOFs (main.f90:76-79), 2*nstep doubles.
 * Returns 0 or a negative status. */
int sdgo_run(double* q, double* q0, double* dqdt, const double* u,
             const double* v, const double* w, const double* D1D,
             const double* D1D_tr, const double* Lift, const int* VMapM,
             const int* VMapP, const double* normal_fn, const double* Escale,
             const double* Fscale, const int* halo_src_map, int Nq, int Ne,
             int NeA, int NhaloNode, double dt, int nstep, int opt,
             double* minmax);

/* Sine initial condition of main.f90:146-157: q = sin(2 pi x) sin(2 pi y)
 * sin(2 pi z) and constant velocity, over owned DOFs. */
void sdgo_ic_sine(double* q, double* u, double* v, double* w,
                  const double* pos_en, int Np, int Ne, double vx, double vy,
                  double vz);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int sdgo_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
