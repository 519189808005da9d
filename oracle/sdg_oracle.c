/*
 * sdg_oracle.c -- CPU restatement of the SCALE-DG kernel-extraction hot path
 * (advection tendency, DG operators, halo update, SSP-RK3), used ONLY as the
 * oracle of the parity tests and as the timed CPU baseline.  See sdg_oracle.h for the
 * parity status and conventions.  Every function cites the reference
 * file:line it restates; the loop and summation order follow the reference
 * so that results agree to rounding.
 */
#include "sdg_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* mod_common.f90:28-30 */
const double sdgo_rk_a[3] = {0.0, 0.75, 1.0 / 3.0};
const double sdgo_rk_b[3] = {1.0, 0.25, 2.0 / 3.0};

int sdgo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Operator file: three list-directed reads (mod_mesh.f90:253-261).  A
 * list-directed read starts at the next record and, once it has its values,
 * leaves the rest of the last record it touched unread; the next read starts
 * on the following line.  Separators are blanks, commas and line ends;
 * exponents may be written with E or D; "r*c" repeats c r times. */

typedef struct {
  char* buf;
  size_t len;
  size_t pos; /* start of the current record */
} sdgo_reader;

static int sdgo_list_read(sdgo_reader* r, double* out, long n) {
  long got = 0;
  size_t pos = r->pos;
  if (pos >= r->len) return -2;
  while (got < n) {
    /* skip separators, crossing record boundaries as needed */
    while (pos < r->len &&
           (r->buf[pos] == ' ' || r->buf[pos] == '\t' || r->buf[pos] == ',' ||
            r->buf[pos] == '\n' || r->buf[pos] == '\r'))
      pos++;
    if (pos >= r->len) return -2;
    if (r->buf[pos] == '/') return -2; /* slash ends the list early */
    char tok[128];
    size_t t = 0;
    while (pos < r->len && !isspace((unsigned char)r->buf[pos]) &&
           r->buf[pos] != ',' && r->buf[pos] != '/') {
      if (t + 1 >= sizeof(tok)) return -2;
      char c = r->buf[pos++];
      tok[t++] = (c == 'D' || c == 'd') ? 'E' : c;
    }
    tok[t] = '\0';
    long rep = 1;
    char* val = tok;
    char* star = strchr(tok, '*');
    if (star) {
      *star = '\0';
      char* endp;
      rep = strtol(tok, &endp, 10);
      if (*endp != '\0' || rep <= 0) return -2;
      val = star + 1;
    }
    char* endp;
    double x = strtod(val, &endp);
    if (endp == val || *endp != '\0') return -2;
    for (long k = 0; k < rep && got < n; k++) out[got++] = x;
  }
  /* the next read starts after the record that held the last value */
  while (pos < r->len && r->buf[pos] != '\n') pos++;
  if (pos < r->len) pos++;
  r->pos = pos;
  return 0;
}

int sdgo_read_operator_file(const char* path, int p, double* x1D, double* D1D,
                            double* D1D_tr, double* Lift) {
  FILE* fp = fopen(path, "rb");
  if (!fp) return -1;
  fseek(fp, 0, SEEK_END);
  long len = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  if (len <= 0) {
    fclose(fp);
    return -2;
  }
  char* buf = (char*)malloc((size_t)len + 1);
  if (!buf) {
    fclose(fp);
    return -3;
  }
  size_t rd = fread(buf, 1, (size_t)len, fp);
  fclose(fp);
  buf[rd] = '\0';
  sdgo_reader r = {buf, rd, 0};
  const int Nq = p + 1;
  int st = sdgo_list_read(&r, x1D, Nq);
  if (!st) st = sdgo_list_read(&r, D1D, (long)Nq * Nq);
  if (!st) st = sdgo_list_read(&r, Lift, 6L * Nq * Nq * Nq);
  free(buf);
  if (st) return st;
  if (D1D_tr) /* D1D_tr = transpose(D1D), mod_mesh.f90:263 */
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++) D1D_tr[i + j * Nq] = D1D[j + i * Nq];
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Face node tables, mod_mesh.f90:265-324. */
void sdgo_fmask(int p, int* Fmask) {
  const int Nq = p + 1, Nq2 = Nq * Nq, Nfp = Nq2;
  int fp;
  fp = 0; /* 1: -y */
  for (int k = 1; k <= Nq; k++)
    for (int i = 1; i <= Nq; i++) Fmask[fp++ + 0 * Nfp] = i + (k - 1) * Nq2;
  fp = 0; /* 2: +x */
  for (int k = 1; k <= Nq; k++)
    for (int j = 1; j <= Nq; j++)
      Fmask[fp++ + 1 * Nfp] = Nq + (j - 1) * Nq + (k - 1) * Nq2;
  fp = 0; /* 3: +y */
  for (int k = 1; k <= Nq; k++)
    for (int i = 1; i <= Nq; i++)
      Fmask[fp++ + 2 * Nfp] = i + (Nq - 1) * Nq + (k - 1) * Nq2;
  fp = 0; /* 4: -x */
  for (int k = 1; k <= Nq; k++)
    for (int j = 1; j <= Nq; j++)
      Fmask[fp++ + 3 * Nfp] = 1 + (j - 1) * Nq + (k - 1) * Nq2;
  fp = 0; /* 5: -z */
  for (int j = 1; j <= Nq; j++)
    for (int i = 1; i <= Nq; i++) Fmask[fp++ + 4 * Nfp] = i + (j - 1) * Nq;
  fp = 0; /* 6: +z */
  for (int j = 1; j <= Nq; j++)
    for (int i = 1; i <= Nq; i++)
      Fmask[fp++ + 5 * Nfp] = i + (j - 1) * Nq + (Nq - 1) * Nq2;
}

int sdgo_nhalo(int NeX, int NeY, int NeZ) {
  return 2 * (NeY * NeZ + NeX * NeZ + NeX * NeY); /* mod_mesh.f90:97 */
}

/* elem_id, mod_mesh.f90:486-493 (1-based) */
static int sdgo_elem_id(int i, int j, int k, int NeX, int NeY) {
  return i + (j - 1) * NeX + (k - 1) * NeX * NeY;
}

/* eval_neighbor_element, mod_mesh.f90:407-483 */
static void sdgo_neighbor(int i, int j, int k, int f, int NeX, int NeY,
                          int NeZ, int* keP, int* oppface, int* is_boundary) {
  *is_boundary = 0;
  switch (f) {
    case 1:
      *oppface = 3;
      if (j > 1) *keP = sdgo_elem_id(i, j - 1, k, NeX, NeY);
      else { *keP = sdgo_elem_id(i, NeY, k, NeX, NeY); *is_boundary = 1; }
      break;
    case 2:
      *oppface = 4;
      if (i < NeX) *keP = sdgo_elem_id(i + 1, j, k, NeX, NeY);
      else { *keP = sdgo_elem_id(1, j, k, NeX, NeY); *is_boundary = 1; }
      break;
    case 3:
      *oppface = 1;
      if (j < NeY) *keP = sdgo_elem_id(i, j + 1, k, NeX, NeY);
      else { *keP = sdgo_elem_id(i, 1, k, NeX, NeY); *is_boundary = 1; }
      break;
    case 4:
      *oppface = 2;
      if (i > 1) *keP = sdgo_elem_id(i - 1, j, k, NeX, NeY);
      else { *keP = sdgo_elem_id(NeX, j, k, NeX, NeY); *is_boundary = 1; }
      break;
    case 5:
      *oppface = 6;
      if (k > 1) *keP = sdgo_elem_id(i, j, k - 1, NeX, NeY);
      else { *keP = sdgo_elem_id(i, j, NeZ, NeX, NeY); *is_boundary = 1; }
      break;
    default:
      *oppface = 5;
      if (k < NeZ) *keP = sdgo_elem_id(i, j, k + 1, NeX, NeY);
      else { *keP = sdgo_elem_id(i, j, 1, NeX, NeY); *is_boundary = 1; }
      break;
  }
}

/* mesh_setup, mod_mesh.f90:74-193, with set_element_position (:332-353)
 * and set_face_geometry (:356-397). */
void sdgo_mesh_setup(int NeX, int NeY, int NeZ, int p, double Lx, double Ly,
                     double Lz, const double* x1D, int* VMapM, int* VMapP,
                     double* normal_fn, double* Escale, double* Fscale,
                     double* pos_en, int* halo_src_map) {
  const int Nq = p + 1, Np = Nq * Nq * Nq, Nfp = Nq * Nq, NfpTot = 6 * Nfp;
  const long Ne = (long)NeX * NeY * NeZ;
  int* Fmask = (int*)malloc(sizeof(int) * (size_t)Nfp * 6);
  sdgo_fmask(p, Fmask);
  const double dx = Lx / (double)NeX, dy = Ly / (double)NeY,
               dz = Lz / (double)NeZ;
  const double fsc[6] = {2.0 / dy, 2.0 / dx, 2.0 / dy, 2.0 / dx, 2.0 / dz,
                         2.0 / dz};
  const int naxis[6] = {1, 0, 1, 0, 2, 2};
  const double nsign[6] = {-1.0, 1.0, 1.0, -1.0, -1.0, 1.0};

#pragma omp parallel for collapse(3) schedule(static)
  for (int k = 1; k <= NeZ; k++)
    for (int j = 1; j <= NeY; j++)
      for (int i = 1; i <= NeX; i++) {
        const long ke = sdgo_elem_id(i, j, k, NeX, NeY);
        const long e0 = ke - 1;
        const double xc = ((double)i - 0.5) * dx;
        const double yc = ((double)j - 0.5) * dy;
        const double zc = ((double)k - 0.5) * dz;
        if (pos_en)
          for (int kk = 0; kk < Nq; kk++)
            for (int jj = 0; jj < Nq; jj++)
              for (int ii = 0; ii < Nq; ii++) {
                const long n = ii + jj * Nq + kk * Nq * Nq;
                pos_en[n + e0 * Np + 0 * Np * Ne] = xc + 0.5 * dx * x1D[ii];
                pos_en[n + e0 * Np + 1 * Np * Ne] = yc + 0.5 * dy * x1D[jj];
                pos_en[n + e0 * Np + 2 * Np * Ne] = zc + 0.5 * dz * x1D[kk];
              }
        if (Escale)
          for (int n = 0; n < Np; n++) {
            Escale[n + e0 * Np + 0 * Np * Ne] = 2.0 / dx;
            Escale[n + e0 * Np + 1 * Np * Ne] = 2.0 / dy;
            Escale[n + e0 * Np + 2 * Np * Ne] = 2.0 / dz;
          }
        for (int f = 0; f < 6; f++)
          for (int fp = 0; fp < Nfp; fp++) {
            const long m = f * Nfp + fp + e0 * NfpTot;
            if (normal_fn)
              for (int d = 0; d < 3; d++)
                normal_fn[m + d * NfpTot * Ne] = (d == naxis[f]) ? nsign[f] : 0.0;
            if (Fscale) Fscale[m] = fsc[f];
          }
        for (int f = 1; f <= 6; f++) {
          int keP, opp, bnd;
          sdgo_neighbor(i, j, k, f, NeX, NeY, NeZ, &keP, &opp, &bnd);
          for (int fp = 0; fp < Nfp; fp++) {
            const long m = (f - 1) * Nfp + fp + e0 * NfpTot;
            if (VMapM) VMapM[m] = Fmask[fp + (f - 1) * Nfp] + (int)(e0 * Np);
            if (!bnd && VMapP)
              VMapP[m] = Fmask[fp + (opp - 1) * Nfp] + (keP - 1) * Np;
          }
        }
      }

  /* serial halo-slot assignment, mod_mesh.f90:171-190 */
  long ibuf = 0;
  for (int k = 1; k <= NeZ; k++)
    for (int j = 1; j <= NeY; j++)
      for (int i = 1; i <= NeX; i++) {
        const long ke = sdgo_elem_id(i, j, k, NeX, NeY);
        for (int f = 1; f <= 6; f++) {
          int keP, opp, bnd;
          sdgo_neighbor(i, j, k, f, NeX, NeY, NeZ, &keP, &opp, &bnd);
          for (int fp = 0; fp < Nfp; fp++) {
            if (bnd) {
              ibuf++;
              if (VMapP)
                VMapP[(f - 1) * Nfp + fp + (ke - 1) * NfpTot] =
                    (int)(Np * Ne + ibuf);
              if (halo_src_map)
                halo_src_map[ibuf - 1] =
                    Fmask[fp + (opp - 1) * Nfp] + (keP - 1) * Np;
            }
          }
        }
      }
  free(Fmask);
}

/* update_halo, mod_mesh.f90:209-221 */
void sdgo_update_halo(double* f, const int* halo_src_map, int Np, int Ne,
                      int NhaloNode) {
  const long base = (long)Np * Ne;
  for (long ibuf = 0; ibuf < NhaloNode; ibuf++)
    f[base + ibuf] = f[halo_src_map[ibuf] - 1];
}

/* cal_elembnd_flux, mod_advect3d_eq.f90:89-142 */
void sdgo_cal_elembnd_flux(double* flux, const double* q, const double* u,
                           const double* v, const double* w, const int* VMapM,
                           const int* VMapP, const double* normal_fn,
                           const double* Fscale, int Np, int NfpTot, int Ne,
                           int NeA) {
  (void)Np;
  (void)NeA;
  const long NT = (long)NfpTot * Ne;
#pragma omp parallel for schedule(static)
  for (long ke = 0; ke < Ne; ke++) {
    for (long m = ke * NfpTot; m < (ke + 1) * NfpTot; m++) {
      const long iM = VMapM[m] - 1, iP = VMapP[m] - 1;
      const double n1 = normal_fn[m], n2 = normal_fn[m + NT],
                   n3 = normal_fn[m + 2 * NT];
      const double qM = q[iM], qP = q[iP];
      const double VelM = u[iM] * n1 + v[iM] * n2 + w[iM] * n3;
      const double VelP = u[iP] * n1 + v[iP] * n2 + w[iP] * n3;
      const double alpha = 0.5 * fabs(VelP + VelM);
      flux[m] = 0.5 * Fscale[m] * (qP * VelP - qM * VelM - alpha * (qP - qM));
    }
  }
}

/* Partial-sum split used by the OPT1 kernels for p>7:
 * np_div3 = round((p+1)/3.0), mod_dg_optr_kernel_opt1.F90.erb:42-44. */
static int sdgo_np_div3(int Nq) {
  return (int)floor((double)Nq / 3.0 + 0.5);
}

/* Contraction of one line: sum_l a[l*sa] * b[l*sb] in GENERAL order
 * (mod_dg_optr_kernel.f90:216-256: start from zero, add l = 1..Nq) or in the
 * OPT1 order (erb:249-273: plain left-to-right sum for p<=7, three partial
 * sums tmp1+tmp2+tmp3 for p>7).  The product operand order follows each
 * branch; IEEE multiplication is commutative so it does not change the
 * result. */
static double sdgo_line(const double* a, long sa, const double* b, long sb,
                        int Nq, int opt) {
  if (opt == SDGO_OPT1 && Nq - 1 > 7) {
    const int d3 = sdgo_np_div3(Nq);
    double t1 = a[0] * b[0];
    for (int l = 1; l < d3; l++) t1 = t1 + a[l * sa] * b[l * sb];
    double t2 = a[d3 * sa] * b[d3 * sb];
    for (int l = d3 + 1; l < 2 * d3; l++) t2 = t2 + a[l * sa] * b[l * sb];
    double t3 = a[2 * d3 * sa] * b[2 * d3 * sb];
    for (int l = 2 * d3 + 1; l < Nq; l++) t3 = t3 + a[l * sa] * b[l * sb];
    return t1 + t2 + t3;
  }
  if (opt == SDGO_OPT1) {
    double s = a[0] * b[0];
    for (int l = 1; l < Nq; l++) s = s + a[l * sa] * b[l * sb];
    return s;
  }
  double s = 0.0;
  for (int l = 0; l < Nq; l++) s = s + a[l * sa] * b[l * sb];
  return s;
}

/* tensorprod_divlike_dirXYZ, mod_dg_optr_kernel.f90:197-258 (GENERAL) and
 * element_operation_kernel_matvec_divlike_dirXYZ_P<p> (erb:228-344, OPT1). */
void sdgo_divlike(double* out_x, double* out_y, double* out_z, const double* D,
                  const double* D_tr, const double* in_x, const double* in_y,
                  const double* in_z, int Nq, int opt) {
  const long Nq2 = (long)Nq * Nq;
  /* x: out_x(i,jk) = sum_l Mat(i,l) * in_x(l,jk) */
  for (long jk = 0; jk < Nq2; jk++)
    for (int i = 0; i < Nq; i++)
      out_x[i + jk * Nq] = sdgo_line(D + i, Nq, in_x + jk * Nq, 1, Nq, opt);
  /* y: out_y(i,j,k) = sum_l in_y(i,l,k) * Mat_tr(l,j) */
  for (int k = 0; k < Nq; k++)
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++)
        out_y[i + j * Nq + k * Nq2] =
            sdgo_line(in_y + i + k * Nq2, Nq, D_tr + (long)j * Nq, 1, Nq, opt);
  /* z: out_z(i,j,k) = sum_l in_z(i,j,l) * Mat_tr(l,k) */
  for (int k = 0; k < Nq; k++)
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++)
        out_z[i + j * Nq + k * Nq2] =
            sdgo_line(in_z + i + j * Nq, Nq2, D_tr + (long)k * Nq, 1, Nq, opt);
}

/* element_operation_kernel_matvec_gradlike_dirXYZ_P<p>
 * (mod_dg_optr_kernel_opt1.F90.erb:166-219): x, y, z contractions of one
 * field, each a running sum from the l = 1 product (the template has no
 * three-way split).  The template's z direction begins with
 * vec_in(i,1,k)*Mat_tr(1,j) (erb:209), a typo for vec_in(i,j,1)*Mat_tr(1,k);
 * this restatement uses the consistent sum over l of vec_in(i,j,l) *
 * Mat_tr(l,k). */
static double sdgo_line_run(const double* a, long sa, const double* b, long sb, int Nq) {
  double s = a[0] * b[0];
  for (int l = 1; l < Nq; l++) s = s + a[l * sa] * b[l * sb];
  return s;
}

void sdgo_gradlike(double* out_x, double* out_y, double* out_z, const double* D,
                   const double* D_tr, const double* in, int Nq) {
  const long Nq2 = (long)Nq * Nq;
  for (long jk = 0; jk < Nq2; jk++)
    for (int i = 0; i < Nq; i++)
      out_x[i + jk * Nq] = sdgo_line_run(D + i, Nq, in + jk * Nq, 1, Nq);
  for (int k = 0; k < Nq; k++)
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++) {
        out_y[i + j * Nq + k * Nq2] =
            sdgo_line_run(in + i + k * Nq2, Nq, D_tr + (long)j * Nq, 1, Nq);
        out_z[i + j * Nq + k * Nq2] =
            sdgo_line_run(in + i + j * Nq, Nq2, D_tr + (long)k * Nq, 1, Nq);
      }
}

/* element_operation_kernel_matvec_divlike_dirXYZ_var5_P<p> (erb:347-465):
 * five variables, (Nq,Nq,Nq,5) per array, each the OPT1-order divlike.  The
 * template's y output index j + (kv-1)*5*Nq (erb:400) lies outside
 * vec_out_y for kv > 1; the output here is vec_out_y(i,j,k,v), the layout of
 * the x and z outputs. */
void sdgo_divlike_var5(double* out_x, double* out_y, double* out_z, const double* D,
                       const double* D_tr, const double* in_x, const double* in_y,
                       const double* in_z, int Nq) {
  const long Np = (long)Nq * Nq * Nq;
  for (int v = 0; v < 5; v++)
    sdgo_divlike(out_x + v * Np, out_y + v * Np, out_z + v * Np, D, D_tr, in_x + v * Np,
                 in_y + v * Np, in_z + v * Np, Nq, SDGO_OPT1);
}

/* tensorprod_Lift_hexahedral, mod_dg_optr_kernel.f90:262-288 */
void sdgo_lift(double* out, const double* Lift, const double* in, int Nq) {
  const long Nq2 = (long)Nq * Nq, Np = Nq2 * Nq;
  for (int k = 0; k < Nq; k++)
    for (int j = 0; j < Nq; j++)
      for (int i = 0; i < Nq; i++) {
        const long n = i + j * Nq + k * Nq2;
        out[n] = Lift[n + 0 * Np] * in[i + k * Nq + 0 * Nq2] +
                 Lift[n + 1 * Np] * in[j + k * Nq + 1 * Nq2] +
                 Lift[n + 2 * Np] * in[i + k * Nq + 2 * Nq2] +
                 Lift[n + 3 * Np] * in[j + k * Nq + 3 * Nq2] +
                 Lift[n + 4 * Np] * in[i + j * Nq + 4 * Nq2] +
                 Lift[n + 5 * Np] * in[i + j * Nq + 5 * Nq2];
      }
}

/* cal_dqdt, mod_advect3d_eq.f90:146-201 */
void sdgo_cal_dqdt(double* dqdt, const double* q, const double* u,
                   const double* v, const double* w, const double* flux_bnd,
                   const double* D1D, const double* D1D_tr,
                   const double* Lift, const double* Escale, int Nq, int Np,
                   int NfpTot, int Ne, int NeA, int opt) {
  (void)NeA;
  const long NpNe = (long)Np * Ne;
#pragma omp parallel
  {
    double* buf = (double*)malloc(sizeof(double) * 7 * (size_t)Np);
    double *fx = buf, *fy = buf + Np, *fz = buf + 2 * Np, *dx = buf + 3 * Np,
           *dy = buf + 4 * Np, *dz = buf + 5 * Np, *lb = buf + 6 * Np;
#pragma omp for schedule(static)
    for (long ke = 0; ke < Ne; ke++) {
      const long o = ke * Np;
      for (int n = 0; n < Np; n++) {
        fx[n] = q[o + n] * u[o + n];
        fy[n] = q[o + n] * v[o + n];
        fz[n] = q[o + n] * w[o + n];
      }
      sdgo_divlike(dx, dy, dz, D1D, D1D_tr, fx, fy, fz, Nq, opt);
      sdgo_lift(lb, Lift, flux_bnd + ke * NfpTot, Nq);
      for (int n = 0; n < Np; n++)
        dqdt[o + n] = -(Escale[o + n] * dx[n] + Escale[o + n + NpNe] * dy[n] +
                        Escale[o + n + 2 * NpNe] * dz[n] + lb[n]);
    }
    free(buf);
  }
}

/* advect3d_eq_cal_tend, mod_advect3d_eq.f90:41-85 */
int sdgo_cal_tend(double* dqdt, const double* q, const double* u,
                  const double* v, const double* w, const double* D1D,
                  const double* D1D_tr, const double* Lift, const int* VMapM,
                  const int* VMapP, const double* normal_fn,
                  const double* Escale, const double* Fscale, int Nq, int Np,
                  int NfpTot, int Ne, int NeA, int opt) {
  double* ebnd = (double*)malloc(sizeof(double) * (size_t)NfpTot * Ne);
  if (!ebnd) return -3;
  sdgo_cal_elembnd_flux(ebnd, q, u, v, w, VMapM, VMapP, normal_fn, Fscale, Np,
                        NfpTot, Ne, NeA);
  sdgo_cal_dqdt(dqdt, q, u, v, w, ebnd, D1D, D1D_tr, Lift, Escale, Nq, Np,
                NfpTot, Ne, NeA, opt);
  free(ebnd);
  return 0;
}

/* RK combine over owned elements, main.f90:68-73 */
void sdgo_rk_stage(double* q, const double* q0, const double* dqdt, int Np,
                   int Ne, int stage, double dt) {
  const double a = sdgo_rk_a[stage], b = sdgo_rk_b[stage];
  const long n = (long)Np * Ne;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) q[i] = a * q0[i] + b * (q[i] + dt * dqdt[i]);
}

/* time loop, main.f90:51-80 */
int sdgo_run(double* q, double* q0, double* dqdt, const double* u,
             const double* v, const double* w, const double* D1D,
             const double* D1D_tr, const double* Lift, const int* VMapM,
             const int* VMapP, const double* normal_fn, const double* Escale,
             const double* Fscale, const int* halo_src_map, int Nq, int Ne,
             int NeA, int NhaloNode, double dt, int nstep, int opt,
             double* minmax) {
  const int Np = Nq * Nq * Nq, NfpTot = 6 * Nq * Nq;
  const long nown = (long)Np * Ne;
  for (int istep = 0; istep < nstep; istep++) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < nown; i++) q0[i] = q[i];
    for (int stage = 0; stage < 3; stage++) {
      sdgo_update_halo(q, halo_src_map, Np, Ne, NhaloNode);
      int st = sdgo_cal_tend(dqdt, q, u, v, w, D1D, D1D_tr, Lift, VMapM, VMapP,
                             normal_fn, Escale, Fscale, Nq, Np, NfpTot, Ne,
                             NeA, opt);
      if (st) return st;
      sdgo_rk_stage(q, q0, dqdt, Np, Ne, stage, dt);
    }
    if (minmax) {
      double mn = q[0], mx = q[0];
      for (long i = 1; i < nown; i++) {
        if (q[i] < mn) mn = q[i];
        if (q[i] > mx) mx = q[i];
      }
      minmax[2 * istep] = mn;
      minmax[2 * istep + 1] = mx;
    }
  }
  return 0;
}

/* initial condition, main.f90:144-157 (PI = 4 atan(1), mod_common.f90:25) */
void sdgo_ic_sine(double* q, double* u, double* v, double* w,
                  const double* pos_en, int Np, int Ne, double vx, double vy,
                  double vz) {
  const double PI = 4.0 * atan(1.0);
  const long n = (long)Np * Ne;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    q[i] = sin(2.0 * PI * pos_en[i]) * sin(2.0 * PI * pos_en[i + n]) *
           sin(2.0 * PI * pos_en[i + 2 * n]);
    u[i] = vx;
    v[i] = vy;
    w[i] = vz;
  }
}
