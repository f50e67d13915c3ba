/*
 * luxum_oracle.c -- CPU restatement of Luxum's time-stepping path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU engine is compared against;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs load it.
 * The engine never links, loads or calls it.
 *
 * PARITY UNPINNED: the reference cannot be built here (it needs blitz++, yaml-cpp 0.3,
 * MPI and parallel HDF5, none of which are installed) and it ships no tests, golden
 * vectors or fixtures with known outputs.  This restatement follows the reference's code
 * line by line (same expressions, same evaluation order, same loop nests and OpenMP
 * schedule, FP64 throughout, no FMA contraction: build with -ffp-contract=off) and cites
 * the file:line of every piece it restates, so that a reader can check it by eye.
 *
 * Layout: every field component is a dense C-order array of its staggered extents
 * (field.cc:58-77), like the reference's blitz arrays; psi and curl arrays are full-grid
 * as in the reference drivers.  Single rank: local = global (grid.cc:75-93 with
 * npX = npY = 1), so global_to_local is the identity and there is no halo exchange.
 *
 * Additions the reference does not have (used by the engine's extra features and by the
 * parity tests; each is marked "extension"): per-component Cb arrays in every driver,
 * point probes, a Gaussian-pulsed additive point source, the textbook CPML b sign.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/luxum.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
  double* a;
  int n0, n1, n2;
} arr3;

#define A3(f, i, j, k) ((f).a[((size_t)(i) * (size_t)(f).n1 + (size_t)(j)) * (size_t)(f).n2 + (size_t)(k)])

typedef struct {
  arr3 x, y, z;
  int face; /* isFaceCentered */
} vf;

/* extension: running-DFT plane monitor (see lx_sim_add_dft_plane in include/luxum.h) */
typedef struct {
  int axis, index, nfreq, every, na, nb;
  int comp[4];
  double* omega;
  double* acc; /* [nfreq][4][na*nb][2] */
} ox_dft;

#define OX_MAX_DFT 16

typedef struct ox_sim {
  lx_params p;
  int planar, pml, threads;
  int Nx, Ny, Nz; /* local_colloq_x/y/z (grid.cc:83-93) */
  /* maxwell members (maxwell.h:60-215) */
  double epsilon0, mew0, S, c, dt, dx, dy, dz, sigma, init;
  double a_max, k_max, m_pml, ma_pml, sigma_optimal, sigma_max, d_pml;
  double H_x_dir, H_y_dir, H_z_dir, E_x_dir, E_y_dir, E_z_dir, kx, ky, kz;
  int p1, q1, r1, p2, q2, r2;
  int start_x, start_y, start_z, end_x, end_y, end_z;
  int amp_source, omega_source, Nx_source, Ny_source, Nz_source;
  /* state */
  vf E, H, Cb, Ecurl, Hcurl, Ecurl1, Ecurl2, Hcurl1, Hcurl2, psi_E1, psi_E2, psi_H1, psi_H2;
  arr3 Etotal;
  double *k_e[3], *k_h[3], *b_e[3], *b_h[3], *c_e[3], *c_h[3];
  double local_max;
  int t;
  /* probes (extension) */
  int nprobes, probe_cap, probe_rows;
  int* probe_ijk;
  double* probe_buf;
  /* DFT planes (extension) */
  int ndft;
  ox_dft dft[OX_MAX_DFT];
} ox_sim;

void ox_destroy(struct ox_sim* s);

/* sizeof(lx_params) as this compiler lays it out (checked against the ctypes mirror). */
size_t ox_params_size(void) { return sizeof(lx_params); }

/* ------------------------------------------------------------------ allocation */

static int arr_alloc(arr3* f, int n0, int n1, int n2) {
  f->n0 = n0 > 0 ? n0 : 0;
  f->n1 = n1 > 0 ? n1 : 0;
  f->n2 = n2 > 0 ? n2 : 0;
  size_t n = (size_t)f->n0 * f->n1 * f->n2;
  f->a = (double*)calloc(n ? n : 1, sizeof(double)); /* zero init: field.cc:78-85 */
  return f->a ? 0 : -1;
}

static void arr_free(arr3* f) {
  free(f->a);
  f->a = NULL;
}

/* vfield::vfield vfield.cc:58-87 -> field::field field.cc:58-92 (extent - 1 per staggered axis). */
static int vf_alloc(ox_sim* s, vf* v, int face) {
  int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz, rc = 0;
  v->face = face;
  memset(&v->x, 0, sizeof(arr3));
  memset(&v->y, 0, sizeof(arr3));
  memset(&v->z, 0, sizeof(arr3));
  if (s->planar) {
    if (face) {
      rc |= arr_alloc(&v->x, Nx, Ny, Nz - 1); /* field(grid,false,false,true) vfield.cc:64 */
      rc |= arr_alloc(&v->z, Nx - 1, Ny, Nz); /* field(grid,true,false,false) vfield.cc:66 */
    } else {
      rc |= arr_alloc(&v->y, Nx, Ny, Nz); /* field(grid,false,false,false) vfield.cc:70 */
    }
  } else {
    if (face) {
      rc |= arr_alloc(&v->x, Nx, Ny - 1, Nz - 1); /* vfield.cc:76 */
      rc |= arr_alloc(&v->y, Nx - 1, Ny, Nz - 1); /* vfield.cc:77 */
      rc |= arr_alloc(&v->z, Nx - 1, Ny - 1, Nz); /* vfield.cc:78 */
    } else {
      rc |= arr_alloc(&v->x, Nx - 1, Ny, Nz); /* vfield.cc:81 */
      rc |= arr_alloc(&v->y, Nx, Ny - 1, Nz); /* vfield.cc:82 */
      rc |= arr_alloc(&v->z, Nx, Ny, Nz - 1); /* vfield.cc:83 */
    }
  }
  return rc;
}

static void vf_free(vf* v) {
  arr_free(&v->x);
  arr_free(&v->y);
  arr_free(&v->z);
}

/* ------------------------------------------------------------------ profiles */

/* Shared head of sigma_fn/k_fn/a_fn (maxwell.cc:997-1035 and the copies at :1058-1096,
 * :1121-1159): per-axis spacing, global N, and the position array temp = index (+0.5 for H). */
static int prof_axis(const ox_sim* s, int dim, double* delta, int* N, int* N_local) {
  if (dim == 0) {
    *delta = s->p.dx; *N_local = s->Nx; *N = s->p.Nx;
  } else if (dim == 1) {
    *delta = s->p.dy; *N_local = s->Ny; *N = s->p.Ny;
  } else if (dim == 2) {
    *delta = s->p.dz; *N_local = s->Nz; *N = s->p.Nz;
  } else {
    return -1;
  }
  return 0;
}

static double prof_pos(int i, int is_E) { return is_E ? (double)(i + 0) : ((double)i + 0.5) + 0; }

/* maxwell::sigma_fn maxwell.cc:997-1042 (w has N_local entries for E, N_local-1 for H). */
static void sigma_fn(const ox_sim* s, int dim, int is_E, double* w) {
  double delta; int N, N_local;
  prof_axis(s, dim, &delta, &N, &N_local);
  int n = is_E ? N_local : N_local - 1;
  double d = s->d_pml / delta; /* :1037 */
  for (int i = 0; i < n; i++) {
    double temp = prof_pos(i, is_E);
    double w0 = 0.0; /* :1038 */
    /* :1039 */
    w0 = (double)(temp <= (d - 1)) * pow((((d - 1) - temp) / (d - 1)), s->m_pml) * s->sigma_max + (double)(temp > (d - 1)) * w0;
    /* :1040 */
    w0 = (double)(temp >= (N - d)) * pow((temp - N + d) / (d - 1), s->m_pml) * s->sigma_max + (double)(temp < (N - d)) * w0;
    w[i] = w0;
  }
}

/* maxwell::k_fn maxwell.cc:1058-1105 */
static void k_fn(const ox_sim* s, int dim, int is_E, double* w) {
  double delta; int N, N_local;
  prof_axis(s, dim, &delta, &N, &N_local);
  int n = is_E ? N_local : N_local - 1;
  double d = s->d_pml / delta; /* :1099 */
  for (int i = 0; i < n; i++) {
    double temp = prof_pos(i, is_E);
    double w0 = 1; /* :1100 */
    /* :1101 */
    w0 = (double)(temp <= (d - 1)) * (pow((((d - 1) - temp) / (d - 1)), s->m_pml) * (s->k_max - 1) + 1) + (double)(temp > (d - 1)) * w0;
    /* :1102 */
    w0 = (double)(temp >= (N - d)) * (pow((temp - N + d) / (d - 1), s->m_pml) * (s->k_max - 1) + 1) + (double)(temp < (N - d)) * w0;
    w[i] = w0;
  }
}

/* maxwell::a_fn maxwell.cc:1121-1167 */
static void a_fn(const ox_sim* s, int dim, int is_E, double* w) {
  double delta; int N, N_local;
  prof_axis(s, dim, &delta, &N, &N_local);
  int n = is_E ? N_local : N_local - 1;
  double d = s->d_pml / delta; /* :1162 */
  for (int i = 0; i < n; i++) {
    double temp = prof_pos(i, is_E);
    double w0 = 0.0; /* :1163 */
    /* :1164 */
    w0 = (double)(temp <= (d - 1)) * pow((temp / (d - 1)), s->ma_pml) * s->a_max + (double)(temp > (d - 1)) * w0;
    /* :1165 */
    w0 = (double)(temp >= (N - d)) * pow((N - 1 - temp) / (d - 1), s->ma_pml) * s->a_max + (double)(temp < (N - d)) * w0;
    w[i] = w0;
  }
}

/* maxwell::b_fn maxwell.cc:1183-1218.  The reference subtracts a (:1215); the extension
 * LX_CPML_STANDARD adds it. */
static void b_fn(const ox_sim* s, int dim, int is_E, double* w) {
  double delta; int N, N_local;
  prof_axis(s, dim, &delta, &N, &N_local);
  int n = is_E ? N_local : N_local - 1;
  double* ts = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double* ta = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double* tk = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  sigma_fn(s, dim, is_E, ts);
  a_fn(s, dim, is_E, ta);
  k_fn(s, dim, is_E, tk);
  for (int i = 0; i < n; i++) {
    if (s->p.cpml_mode == LX_CPML_STANDARD)
      w[i] = exp(-((ts[i] / tk[i] / s->epsilon0) + (ta[i] / s->epsilon0)) * s->dt);
    else
      w[i] = exp(-((ts[i] / tk[i] / s->epsilon0) - (ta[i] / s->epsilon0)) * s->dt); /* :1215 */
  }
  free(ts); free(ta); free(tk);
}

/* maxwell::c_fn maxwell.cc:1234-1280 */
static void c_fn(const ox_sim* s, int dim, int is_E, double* w) {
  double delta; int N, N_local;
  prof_axis(s, dim, &delta, &N, &N_local);
  int n = is_E ? N_local : N_local - 1;
  double* ts = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double* ta = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  double* tk = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  sigma_fn(s, dim, is_E, ts);
  a_fn(s, dim, is_E, ta);
  k_fn(s, dim, is_E, tk);
  b_fn(s, dim, is_E, w); /* :1266 */
  for (int i = 0; i < n; i++) { /* :1271-1278 */
    if (ts[i] == 0) {
      w[i] = 0.0;
    } else {
      w[i] = ts[i] / (ts[i] * tk[i] + pow(tk[i], 2) * ta[i]) * (w[i] - 1);
    }
  }
  free(ts); free(ta); free(tk);
}

/* ------------------------------------------------------------------ set-up */

/* maxwell::plane_wave_initialise maxwell.cc:825-929 for one axis (single rank:
 * colloq_start = 0, colloq_end = N-1 in x/y (grid.cc:75-79), Nz-1 in z (:80)). */
static void pw_clip(int a1, int a2, int cs, int ce, int* st, int* en) {
  if (a1 > ce) {
    *st = -1; *en = -1;
  } else if (a1 >= cs) {
    *st = a1;
    *en = (a2 > ce) ? ce : a2;
  } else {
    if (a2 > ce) { *st = cs; *en = ce; }
    else if (a2 >= cs) { *st = cs; *en = a2; }
    else { *st = -1; *en = -1; }
  }
}

static int ox_validate(const lx_params* p) {
  /* reader::checkData reader.cc:141-162 */
  if (p->npX < 1 || p->npY < 1) return LX_ERR_INVALID;
  if ((p->Nx - 2) % p->npX != 0) return LX_ERR_INVALID;
  if ((p->Ny - 2) % p->npY != 0) return LX_ERR_INVALID;
  if (p->isPlanar && p->Ny != 1) return LX_ERR_INVALID;
  if (p->isPlanar && p->npY != 1) return LX_ERR_INVALID;
  /* ranges the reference reads out of bounds or divides by zero on */
  if (p->Nx < 3 || p->Nz < 3 || (!p->isPlanar && p->Ny < 3)) return LX_ERR_INVALID;
  if (!(p->dx > 0) || !(p->dz > 0) || (!p->isPlanar && !(p->dy > 0)) || !(p->S > 0)) return LX_ERR_INVALID;
  if (p->num_timesteps < 0) return LX_ERR_INVALID;
  if (p->usePW) {
    if (p->x1_pw < 1 || p->x2_pw > p->Nx - 2 || p->x1_pw > p->x2_pw) return LX_ERR_INVALID;
    if (p->z1_pw < 1 || p->z2_pw > p->Nz - 2 || p->z1_pw > p->z2_pw) return LX_ERR_INVALID;
    if (!p->isPlanar && (p->y1_pw < 1 || p->y2_pw > p->Ny - 2 || p->y1_pw > p->y2_pw)) return LX_ERR_INVALID;
    double hx = p->ky_pw * p->Ez_pw - p->kz_pw * p->Ey_pw;
    double hy = p->kz_pw * p->Ex_pw - p->kx_pw * p->Ez_pw;
    double hz = p->kx_pw * p->Ey_pw - p->ky_pw * p->Ex_pw;
    if (hx == 0 && hy == 0 && hz == 0) return LX_ERR_INVALID;
    if (!(p->pw_sigma > 0)) return LX_ERR_INVALID;
  }
  if (p->usePML) {
    double d0 = p->d_pml / p->dx, d2 = p->d_pml / p->dz, d1 = p->isPlanar ? 2.0 : p->d_pml / p->dy;
    if (!(d0 > 1) || !(d1 > 1) || !(d2 > 1)) return LX_ERR_INVALID;
    if (p->sigma_m != floor(p->sigma_m)) return LX_ERR_INVALID; /* pow(negative, non-integer) = NaN in sigma_fn/k_fn */
  }
  if (p->usePS) {
    if (p->isPlanar && p->source_kind == LX_SRC_CW_HARD) return LX_ERR_UNSUPPORTED; /* E->Vz is NULL in planar (vfield.cc:69-71) */
    if (p->source_kind != LX_SRC_CW_HARD && p->source_kind != LX_SRC_PULSE_SOFT) return LX_ERR_INVALID;
    int zext = p->isPlanar ? p->Nz : p->Nz - 1;
    if (p->Nz_source < 0 || p->Nz_source >= zext) return LX_ERR_INVALID; /* z is not range-checked by check_global_limits */
    if (p->source_kind == LX_SRC_PULSE_SOFT && !(p->src_tw > 0)) return LX_ERR_INVALID;
  }
  if ((double)p->Nx * (p->isPlanar ? 1 : p->Ny) * p->Nz > 4.0e9) return LX_ERR_INVALID;
  if (p->precision < LX_PREC_FP64 || p->precision > LX_PREC_FP16S) return LX_ERR_INVALID;
  if (p->monitor_every < 0) return LX_ERR_INVALID;
  return LX_OK;
}

int ox_create(const lx_params* p, ox_sim** out) {
  *out = NULL;
  int rc = ox_validate(p);
  if (rc) return rc;
  ox_sim* s = (ox_sim*)calloc(1, sizeof(ox_sim));
  if (!s) return LX_ERR_OOM;
  s->p = *p;
  s->planar = p->isPlanar != 0;
  s->pml = p->usePML != 0;
  s->threads = p->n_threads > 0 ? p->n_threads : 1;
  /* grid::grid grid.cc:83-93 with npX = npY = 1 */
  s->Nx = (p->Nx - 2) / 1 + 2;
  s->Ny = s->planar ? 1 : (p->Ny - 2) / 1 + 2;
  s->Nz = p->Nz;

  /* maxwell::maxwell maxwell.cc:60-148 */
  s->epsilon0 = 8.85 * pow(10, -12);
  s->mew0 = M_PI * 4 * pow(10, -7);
  s->S = p->S;
  s->c = 1 / pow(s->epsilon0 * s->mew0, 0.5);
  s->dt = s->S * p->dx / s->c;
  s->dx = p->dx;
  s->dy = p->dy;
  s->dz = p->dz;
  s->sigma = p->pw_sigma; /* pow(10,-4)/0.5 by default (:71) */
  s->init = p->off_pw;
  if (s->pml) { /* :78-86 */
    s->a_max = p->a_max;
    s->k_max = p->kappa;
    s->m_pml = p->sigma_m;
    s->ma_pml = p->a_m;
    s->sigma_optimal = 0.8 * (s->m_pml + 1) / s->dx / pow(s->mew0 / s->epsilon0, 0.5);
    s->sigma_max = s->sigma_optimal * p->sigma;
    s->d_pml = p->d_pml;
  }
  if (p->usePW) { /* :87-140 */
    s->E_x_dir = p->Ex_pw;
    s->E_y_dir = p->Ey_pw;
    s->E_z_dir = p->Ez_pw;
    s->kx = p->kx_pw;
    s->ky = p->ky_pw;
    s->kz = p->kz_pw;
    s->H_x_dir = s->ky * s->E_z_dir - s->kz * s->E_y_dir;
    s->H_y_dir = s->kz * s->E_x_dir - s->kx * s->E_z_dir;
    s->H_z_dir = s->kx * s->E_y_dir - s->ky * s->E_x_dir;
    double H_abs = pow(pow(s->H_x_dir, 2) + pow(s->H_y_dir, 2) + pow(s->H_z_dir, 2), 0.5);
    s->H_x_dir = s->H_x_dir / H_abs;
    s->H_y_dir = s->H_y_dir / H_abs;
    s->H_z_dir = s->H_z_dir / H_abs;
    s->p1 = p->x1_pw; s->q1 = p->y1_pw; s->r1 = p->z1_pw;
    s->p2 = p->x2_pw; s->q2 = p->y2_pw; s->r2 = p->z2_pw;
    /* plane_wave_initialise :825-913; planar grids have colloq y range [0,0] (grid.cc:89-93) */
    pw_clip(s->p1, s->p2, 0, s->Nx - 1, &s->start_x, &s->end_x);
    if (s->planar) pw_clip(s->q1, s->q2, 0, 0, &s->start_y, &s->end_y);
    else pw_clip(s->q1, s->q2, 0, s->Ny - 1, &s->start_y, &s->end_y);
    pw_clip(s->r1, s->r2, 0, s->Nz - 1, &s->start_z, &s->end_z);
  }
  if (p->usePS) { /* :141-147 (int members truncate the doubles) */
    s->amp_source = (int)p->amp_source;
    s->omega_source = (int)p->omega_source;
    s->Nx_source = p->Nx_source;
    s->Ny_source = p->Ny_source;
    s->Nz_source = p->Nz_source;
  }

  int arc = 0;
  arc |= vf_alloc(s, &s->E, 0);
  arc |= vf_alloc(s, &s->H, 1);
  arc |= vf_alloc(s, &s->Cb, 0);
  if (s->pml) {
    arc |= vf_alloc(s, &s->Ecurl1, 1);
    arc |= vf_alloc(s, &s->Ecurl2, 1);
    arc |= vf_alloc(s, &s->Hcurl1, 0);
    arc |= vf_alloc(s, &s->Hcurl2, 0);
    arc |= vf_alloc(s, &s->psi_E1, 0);
    arc |= vf_alloc(s, &s->psi_E2, 0);
    arc |= vf_alloc(s, &s->psi_H1, 1);
    arc |= vf_alloc(s, &s->psi_H2, 1);
    for (int d = 0; d < 3; d++) {
      int n = d == 0 ? s->Nx : (d == 1 ? s->Ny : s->Nz);
      if (s->planar && d == 1) continue;
      s->k_e[d] = (double*)calloc((size_t)n, sizeof(double));
      s->b_e[d] = (double*)calloc((size_t)n, sizeof(double));
      s->c_e[d] = (double*)calloc((size_t)n, sizeof(double));
      s->k_h[d] = (double*)calloc((size_t)n, sizeof(double));
      s->b_h[d] = (double*)calloc((size_t)n, sizeof(double));
      s->c_h[d] = (double*)calloc((size_t)n, sizeof(double));
      if (!s->k_e[d] || !s->b_e[d] || !s->c_e[d] || !s->k_h[d] || !s->b_h[d] || !s->c_h[d]) arc = -1;
      else {
        /* two_dim_pml.cc:66-83, three_dim_pml.cc:65-88 */
        k_fn(s, d, 1, s->k_e[d]); k_fn(s, d, 0, s->k_h[d]);
        b_fn(s, d, 1, s->b_e[d]); b_fn(s, d, 0, s->b_h[d]);
        c_fn(s, d, 1, s->c_e[d]); c_fn(s, d, 0, s->c_h[d]);
      }
    }
  } else {
    arc |= vf_alloc(s, &s->Ecurl, 1);
    arc |= vf_alloc(s, &s->Hcurl, 0);
  }
  if (!s->planar) arc |= arr_alloc(&s->Etotal, s->Nx, s->Ny, s->Nz - 1);
  if (arc) {
    ox_destroy(s);
    return LX_ERR_OOM;
  }
  /* Cb = dt/epsilon0 (two_dim.cc:81, two_dim_pml.cc:116, three_dim.cc:54 as an array) */
  arr3* cbs[3] = {&s->Cb.x, &s->Cb.y, &s->Cb.z};
  for (int c = 0; c < 3; c++) {
    size_t n = (size_t)cbs[c]->n0 * cbs[c]->n1 * cbs[c]->n2;
    for (size_t q = 0; q < n; q++) cbs[c]->a[q] = s->dt / s->epsilon0;
  }
  s->local_max = 0.0;
  *out = s;
  return LX_OK;
}

void ox_destroy(ox_sim* s) {
  if (!s) return;
  vf* all[] = {&s->E, &s->H, &s->Cb, &s->Ecurl, &s->Hcurl, &s->Ecurl1, &s->Ecurl2, &s->Hcurl1,
               &s->Hcurl2, &s->psi_E1, &s->psi_E2, &s->psi_H1, &s->psi_H2};
  for (size_t q = 0; q < sizeof(all) / sizeof(all[0]); q++) vf_free(all[q]);
  arr_free(&s->Etotal);
  for (int d = 0; d < 3; d++) {
    free(s->k_e[d]); free(s->b_e[d]); free(s->c_e[d]);
    free(s->k_h[d]); free(s->b_h[d]); free(s->c_h[d]);
  }
  free(s->probe_ijk);
  free(s->probe_buf);
  for (int q = 0; q < s->ndft; q++) {
    free(s->dft[q].omega);
    free(s->dft[q].acc);
  }
  free(s);
}

static arr3* comp_arr(ox_sim* s, int comp) {
  switch (comp) {
    case LX_EX: return &s->E.x;
    case LX_EY: return &s->E.y;
    case LX_EZ: return &s->E.z;
    case LX_HX: return &s->H.x;
    case LX_HY: return &s->H.y;
    case LX_HZ: return &s->H.z;
    case LX_ETOTAL: return s->planar ? NULL : &s->Etotal;
    default: return NULL;
  }
}

int ox_field_shape(ox_sim* s, int comp, int shape[3]) {
  arr3* f = comp_arr(s, comp);
  if (!f) return LX_ERR_INVALID;
  if (!f->a || (size_t)f->n0 * f->n1 * f->n2 == 0 || (s->planar && (comp == LX_EX || comp == LX_EZ || comp == LX_HY))) {
    shape[0] = shape[1] = shape[2] = 0;
    return LX_OK;
  }
  shape[0] = f->n0; shape[1] = f->n1; shape[2] = f->n2;
  return LX_OK;
}

int ox_read_field(ox_sim* s, int comp, double* out, size_t n) {
  int sh[3];
  if (ox_field_shape(s, comp, sh)) return LX_ERR_INVALID;
  size_t m = (size_t)sh[0] * sh[1] * sh[2];
  if (n != m) return LX_ERR_INVALID;
  if (m) memcpy(out, comp_arr(s, comp)->a, m * sizeof(double));
  return LX_OK;
}

int ox_write_field(ox_sim* s, int comp, const double* in, size_t n) {
  int sh[3];
  if (comp > LX_HZ || ox_field_shape(s, comp, sh)) return LX_ERR_INVALID;
  size_t m = (size_t)sh[0] * sh[1] * sh[2];
  if (n != m) return LX_ERR_INVALID;
  if (m) memcpy(comp_arr(s, comp)->a, in, m * sizeof(double));
  return LX_OK;
}

/* Appends component `comp` to the file at `path` as its contiguous C-order doubles: the bytes
 * fileio::writeHDF5 puts in one snapshot dataset (fileio.cc:186-201, H5T_NATIVE_DOUBLE,
 * contiguous layout), without the HDF5 metadata.  Used to time the drivers' snapshot writes
 * in the CPU baseline. */
int ox_append_raw(ox_sim* s, int comp, const char* path) {
  int sh[3];
  if (ox_field_shape(s, comp, sh)) return LX_ERR_INVALID;
  const size_t m = (size_t)sh[0] * sh[1] * sh[2];
  FILE* f = fopen(path, "ab");
  if (!f) return LX_ERR_IO;
  const size_t w = m ? fwrite(comp_arr(s, comp)->a, sizeof(double), m, f) : 0;
  if (fclose(f) != 0 || w != m) return LX_ERR_IO;
  return LX_OK;
}

static arr3* cb_arr(ox_sim* s, int comp) {
  if (comp == LX_EX && !s->planar) return &s->Cb.x;
  if (comp == LX_EY) return &s->Cb.y;
  if (comp == LX_EZ && !s->planar) return &s->Cb.z;
  return NULL;
}

/* extension: Cb arrays in every driver (the reference fixes them, e.g. two_dim_pml.cc:116) */
int ox_set_cb(ox_sim* s, int comp, const double* cb, size_t n) {
  arr3* f = cb_arr(s, comp);
  if (!f || n != (size_t)f->n0 * f->n1 * f->n2) return LX_ERR_INVALID;
  memcpy(f->a, cb, n * sizeof(double));
  return LX_OK;
}

/* three_dim_pml.cc:122-128: Cb = dt / (epsilon0 * (1 + F * scale)) */
int ox_set_material(ox_sim* s, int comp, const double* F, size_t n, double scale) {
  arr3* f = cb_arr(s, comp);
  if (!f || n != (size_t)f->n0 * f->n1 * f->n2) return LX_ERR_INVALID;
  for (size_t q = 0; q < n; q++) {
    double e = s->epsilon0 * (1 + F[q] * scale);
    f->a[q] = s->dt / e;
  }
  return LX_OK;
}

int ox_set_eps_box(ox_sim* s, const int lo[3], const int hi[3], double eps_r) {
  for (int c = 0; c < 3; c++) {
    arr3* f = cb_arr(s, c);
    if (!f) continue;
    for (int i = lo[0]; i < hi[0] && i < f->n0; i++)
      for (int j = lo[1]; j < hi[1] && j < f->n1; j++)
        for (int k = lo[2]; k < hi[2] && k < f->n2; k++)
          if (i >= 0 && j >= 0 && k >= 0) A3(*f, i, j, k) = s->dt / (s->epsilon0 * eps_r);
  }
  return LX_OK;
}

int ox_profile(ox_sim* s, int which, int dim, int is_E, double* out, size_t n) {
  double delta; int N, N_local;
  if (prof_axis(s, dim, &delta, &N, &N_local)) return LX_ERR_INVALID;
  size_t m = (size_t)(is_E ? N_local : N_local - 1);
  if (n != m) return LX_ERR_INVALID;
  switch (which) {
    case 0: sigma_fn(s, dim, is_E, out); break;
    case 1: k_fn(s, dim, is_E, out); break;
    case 2: a_fn(s, dim, is_E, out); break;
    case 3: b_fn(s, dim, is_E, out); break;
    case 4: c_fn(s, dim, is_E, out); break;
    default: return LX_ERR_INVALID;
  }
  return LX_OK;
}

void ox_set_threads(ox_sim* s, int n) { s->threads = n > 0 ? n : 1; }
int ox_timestep(ox_sim* s) { return s->t; }
double ox_max_e2(ox_sim* s) { return s->local_max; }

int ox_set_probes(ox_sim* s, const int* ijk, int nprobes, int cap) {
  free(s->probe_ijk); free(s->probe_buf);
  s->probe_ijk = NULL; s->probe_buf = NULL;
  s->nprobes = 0; s->probe_cap = 0; s->probe_rows = 0;
  if (nprobes <= 0) return LX_OK;
  s->probe_ijk = (int*)malloc(sizeof(int) * 3 * (size_t)nprobes);
  s->probe_buf = (double*)calloc((size_t)nprobes * 6 * (size_t)(cap > 0 ? cap : 1), sizeof(double));
  if (!s->probe_ijk || !s->probe_buf) return LX_ERR_OOM;
  memcpy(s->probe_ijk, ijk, sizeof(int) * 3 * (size_t)nprobes);
  s->nprobes = nprobes;
  s->probe_cap = cap;
  return LX_OK;
}

int ox_read_probes(ox_sim* s, double* out, size_t n, int* rows) {
  size_t m = (size_t)s->probe_rows * s->nprobes * 6;
  *rows = s->probe_rows;
  if (n < m) return LX_ERR_INVALID;
  if (m) memcpy(out, s->probe_buf, m * sizeof(double));
  return LX_OK;
}

/* ------------------------------------------------------------------ curls */

/* vfield::curl_3d vfield.cc:102-174 (E -> face-centred curl, then H -> edge-centred curl) */
static void curl_3d(ox_sim* s, vf* src, vf* curl) {
  int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz, nt = s->threads;
  double dx = s->dx, dy = s->dy, dz = s->dz;
  if (!src->face) {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < Nx; i++)
      for (int j = 0; j < (Ny - 1); j++)
        for (int k = 0; k < (Nz - 1); k++)
          A3(curl->x, i, j, k) = (A3(src->z, i, j + 1, k) - A3(src->z, i, j, k)) / dy - (A3(src->y, i, j, k + 1) - A3(src->y, i, j, k)) / dz;
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int j = 0; j < Ny; j++)
      for (int i = 0; i < (Nx - 1); i++)
        for (int k = 0; k < (Nz - 1); k++)
          A3(curl->y, i, j, k) = (A3(src->x, i, j, k + 1) - A3(src->x, i, j, k)) / dz - (A3(src->z, i + 1, j, k) - A3(src->z, i, j, k)) / dx;
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int k = 0; k < Nz; k++)
      for (int j = 0; j < (Ny - 1); j++)
        for (int i = 0; i < (Nx - 1); i++)
          A3(curl->z, i, j, k) = (A3(src->y, i + 1, j, k) - A3(src->y, i, j, k)) / dx - (A3(src->x, i, j + 1, k) - A3(src->x, i, j, k)) / dy;
  } else {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < (Nx - 1); i++)
      for (int j = 1; j < (Ny - 1); j++)
        for (int k = 1; k < (Nz - 1); k++)
          A3(curl->x, i, j, k) = (A3(src->z, i, j, k) - A3(src->z, i, j - 1, k)) / dy - (A3(src->y, i, j, k) - A3(src->y, i, j, k - 1)) / dz;
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int j = 0; j < (Ny - 1); j++)
      for (int i = 1; i < (Nx - 1); i++)
        for (int k = 1; k < (Nz - 1); k++)
          A3(curl->y, i, j, k) = (A3(src->x, i, j, k) - A3(src->x, i, j, k - 1)) / dz - (A3(src->z, i, j, k) - A3(src->z, i - 1, j, k)) / dx;
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int k = 0; k < (Nz - 1); k++)
      for (int j = 1; j < (Ny - 1); j++)
        for (int i = 1; i < (Nx - 1); i++)
          A3(curl->z, i, j, k) = (A3(src->y, i, j, k) - A3(src->y, i - 1, j, k)) / dx - (A3(src->x, i, j, k) - A3(src->x, i, j - 1, k)) / dy;
  }
}

/* vfield::curl_3d_adv vfield.cc:196-275 (positive part -> curl1, negative part -> curl2) */
static void curl_3d_adv(ox_sim* s, vf* src, vf* c1, vf* c2) {
  int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz, nt = s->threads;
  double dx = s->dx, dy = s->dy, dz = s->dz;
  if (!src->face) {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < Nx; i++)
      for (int j = 0; j < (Ny - 1); j++)
        for (int k = 0; k < (Nz - 1); k++) {
          A3(c1->x, i, j, k) = (A3(src->z, i, j + 1, k) - A3(src->z, i, j, k)) / dy;
          A3(c2->x, i, j, k) = (A3(src->y, i, j, k + 1) - A3(src->y, i, j, k)) / dz;
        }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int j = 0; j < Ny; j++)
      for (int i = 0; i < (Nx - 1); i++)
        for (int k = 0; k < (Nz - 1); k++) {
          A3(c1->y, i, j, k) = (A3(src->x, i, j, k + 1) - A3(src->x, i, j, k)) / dz;
          A3(c2->y, i, j, k) = (A3(src->z, i + 1, j, k) - A3(src->z, i, j, k)) / dx;
        }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int k = 0; k < Nz; k++)
      for (int j = 0; j < (Ny - 1); j++)
        for (int i = 0; i < (Nx - 1); i++) {
          A3(c1->z, i, j, k) = (A3(src->y, i + 1, j, k) - A3(src->y, i, j, k)) / dx;
          A3(c2->z, i, j, k) = (A3(src->x, i, j + 1, k) - A3(src->x, i, j, k)) / dy;
        }
  } else {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < (Nx - 1); i++)
      for (int j = 1; j < (Ny - 1); j++)
        for (int k = 1; k < (Nz - 1); k++) {
          A3(c1->x, i, j, k) = (A3(src->z, i, j, k) - A3(src->z, i, j - 1, k)) / dy;
          A3(c2->x, i, j, k) = (A3(src->y, i, j, k) - A3(src->y, i, j, k - 1)) / dz;
        }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int j = 0; j < (Ny - 1); j++)
      for (int i = 1; i < (Nx - 1); i++)
        for (int k = 1; k < (Nz - 1); k++) {
          A3(c1->y, i, j, k) = (A3(src->x, i, j, k) - A3(src->x, i, j, k - 1)) / dz;
          A3(c2->y, i, j, k) = (A3(src->z, i, j, k) - A3(src->z, i - 1, j, k)) / dx;
        }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int k = 0; k < (Nz - 1); k++)
      for (int j = 1; j < (Ny - 1); j++)
        for (int i = 1; i < (Nx - 1); i++) {
          A3(c1->z, i, j, k) = (A3(src->y, i, j, k) - A3(src->y, i - 1, j, k)) / dx;
          A3(c2->z, i, j, k) = (A3(src->x, i, j, k) - A3(src->x, i, j - 1, k)) / dy;
        }
  }
}

/* vfield::curl_planar vfield.cc:293-328 */
static void curl_planar(ox_sim* s, vf* src, vf* curl) {
  int Nx = s->Nx, Nz = s->Nz, nt = s->threads;
  double dx = s->dx, dz = s->dz;
  if (!src->face) {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < (Nx); i++)
      for (int j = 0; j < (Nz - 1); j++)
        A3(curl->x, i, 0, j) = -(A3(src->y, i, 0, j + 1) - A3(src->y, i, 0, j)) / dz;
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < (Nx - 1); i++)
      for (int j = 0; j < (Nz); j++)
        A3(curl->z, i, 0, j) = (A3(src->y, i + 1, 0, j) - A3(src->y, i, 0, j)) / dx;
  } else {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 1; i < (Nx - 1); i++)
      for (int j = 1; j < (Nz - 1); j++)
        A3(curl->y, i, 0, j) = (A3(src->x, i, 0, j) - A3(src->x, i, 0, j - 1)) / dz - (A3(src->z, i, 0, j) - A3(src->z, i - 1, 0, j)) / dx;
  }
}

/* vfield::curl_planar_adv vfield.cc:350-386 */
static void curl_planar_adv(ox_sim* s, vf* src, vf* c1, vf* c2) {
  int Nx = s->Nx, Nz = s->Nz, nt = s->threads;
  double dx = s->dx, dz = s->dz;
  if (!src->face) {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < (Nx); i++)
      for (int j = 0; j < (Nz - 1); j++)
        A3(c2->x, i, 0, j) = (A3(src->y, i, 0, j + 1) - A3(src->y, i, 0, j)) / dz;
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 0; i < (Nx - 1); i++)
      for (int j = 0; j < (Nz); j++)
        A3(c1->z, i, 0, j) = (A3(src->y, i + 1, 0, j) - A3(src->y, i, 0, j)) / dx;
  } else {
#pragma omp parallel for num_threads(nt) schedule(dynamic)
    for (int i = 1; i < (Nx - 1); i++)
      for (int j = 1; j < (Nz - 1); j++) {
        A3(c1->y, i, 0, j) = (A3(src->x, i, 0, j) - A3(src->x, i, 0, j - 1)) / dz;
        A3(c2->y, i, 0, j) = (A3(src->z, i, 0, j) - A3(src->z, i - 1, 0, j)) / dx;
      }
  }
}

/* ------------------------------------------------------------------ TF/SF */

/* The Gaussian of every plane_wave_execute line: exp(-pow(X,2)/sigma) with
 * X = ((position . k) + init*dx) - (time*c*dt), evaluated in the reference's order. */
#define PW_G(s, X) exp(-pow((X), 2) / (s)->sigma)
#define PW_T(s, tt) ((tt) * (s)->c * (s)->dt)

/* maxwell::plane_wave_execute(vfield*,int) maxwell.cc:194-497 (non-PML drivers) */
static void plane_wave_execute(ox_sim* s, vf* curl, int timestep) {
  double dx = s->dx, dy = s->dy, dz = s->dz, kx = s->kx, ky = s->ky, kz = s->kz, init = s->init, c = s->c, mew0 = s->mew0;
  int p1 = s->p1, p2 = s->p2, q1 = s->q1, q2 = s->q2, r1 = s->r1, r2 = s->r2;
  int sx = s->start_x, ex = s->end_x, sy = s->start_y, ey = s->end_y, sz = s->start_z, ez = s->end_z;
  int xe = s->Nx - 1, ye = s->planar ? 0 : s->Ny - 1, ze = s->Nz - 1;
  double tm = timestep - 0.5, tp = timestep;
  if (s->planar) {
    if (curl->face) {
      if ((p1 - 1) >= 0 && (p1 - 1) <= xe && sz != -1) /* :202-207 */
        for (int k = sz; k <= ez; k++)
          A3(curl->z, p1 - 1, 0, k) = A3(curl->z, p1 - 1, 0, k) + PW_G(s, ((p1 * dx * kx + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      if (p2 >= 0 && p2 <= xe && sz != -1) /* :209-214 */
        for (int k = sz; k <= ez; k++)
          A3(curl->z, p2, 0, k) = A3(curl->z, p2, 0, k) - PW_G(s, ((p2 * dx * kx + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      if ((r1 - 1) >= 0 && (r1 - 1) <= ze && sx != -1) /* :220-225 */
        for (int i = sx; i <= ex; i++)
          A3(curl->x, i, 0, r1 - 1) = A3(curl->x, i, 0, r1 - 1) - PW_G(s, ((i * dx * kx + r1 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
      if (r2 >= 0 && r2 <= ze && sx != -1) /* :227-232 */
        for (int i = sx; i <= ex; i++)
          A3(curl->x, i, 0, r2) = A3(curl->x, i, 0, r2) + PW_G(s, ((i * dx * kx + r2 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
    } else {
      if (p1 >= 0 && p1 <= xe && sz != -1) /* :239-244 */
        for (int k = sz; k <= ez; k++)
          A3(curl->y, p1, 0, k) = A3(curl->y, p1, 0, k) + PW_G(s, (((p1 - 0.5) * dx * kx + k * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_z_dir / dx / c / mew0;
      if (p2 >= 0 && p2 <= xe && sz != -1) /* :246-251 */
        for (int k = sz; k <= ez; k++)
          A3(curl->y, p2, 0, k) = A3(curl->y, p2, 0, k) - PW_G(s, (((p2 + 0.5) * dx * kx + k * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_z_dir / dx / c / mew0;
      if (r1 >= 0 && r1 <= ze && sx != -1) /* :257-262 */
        for (int i = sx; i <= ex; i++)
          A3(curl->y, i, 0, r1) = A3(curl->y, i, 0, r1) - PW_G(s, ((i * dx * kx + (r1 - 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_x_dir / dz / c / mew0;
      if (r2 >= 0 && r2 <= ze && sx != -1) /* :264-269 */
        for (int i = sx; i <= ex; i++)
          A3(curl->y, i, 0, r2) = A3(curl->y, i, 0, r2) + PW_G(s, ((i * dx * kx + (r2 + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_x_dir / dz / c / mew0;
    }
    return;
  }
  if (curl->face) {
    if ((p1 - 1) >= 0 && (p1 - 1) <= xe && sy != -1 && sz != -1) { /* :284-299 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl->z, p1 - 1, j, k) = A3(curl->z, p1 - 1, j, k) - PW_G(s, ((p1 * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->y, p1 - 1, j, k) = A3(curl->y, p1 - 1, j, k) + PW_G(s, ((p1 * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dx;
    }
    if (p2 >= 0 && p2 <= xe && sy != -1 && sz != -1) { /* :300-315 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl->z, p2, j, k) = A3(curl->z, p2, j, k) + PW_G(s, ((p2 * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->y, p2, j, k) = A3(curl->y, p2, j, k) - PW_G(s, ((p2 * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dx;
    }
    if ((q1 - 1) >= 0 && (q1 - 1) <= ye && sx != -1 && sz != -1) { /* :319-334 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl->z, i, q1 - 1, k) = A3(curl->z, i, q1 - 1, k) + PW_G(s, (((i + 0.5) * dx * kx + q1 * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dy;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->x, i, q1 - 1, k) = A3(curl->x, i, q1 - 1, k) - PW_G(s, ((i * dx * kx + q1 * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dy;
    }
    if (q2 >= 0 && q2 <= ye && sx != -1 && sz != -1) { /* :335-350 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl->z, i, q2, k) = A3(curl->z, i, q2, k) - PW_G(s, (((i + 0.5) * dx * kx + q2 * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dy;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->x, i, q2, k) = A3(curl->x, i, q2, k) + PW_G(s, ((i * dx * kx + q2 * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dy;
    }
    if ((r1 - 1) >= 0 && (r1 - 1) <= ze && sx != -1 && sy != -1) { /* :355-370 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl->y, i, j, r1 - 1) = A3(curl->y, i, j, r1 - 1) - PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + r1 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dz;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl->x, i, j, r1 - 1) = A3(curl->x, i, j, r1 - 1) + PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + r1 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
    }
    if (r2 >= 0 && r2 <= ze && sx != -1 && sy != -1) { /* :371-386 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl->y, i, j, r2) = A3(curl->y, i, j, r2) + PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + r2 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dz;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl->x, i, j, r2) = A3(curl->x, i, j, r2) - PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + r2 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
    }
  } else {
    if (p1 >= 0 && p1 <= xe && sy != -1 && sz != -1) { /* :392-407 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl->y, p1, j, k) = A3(curl->y, p1, j, k) + PW_G(s, (((p1 - 0.5) * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dx / c / mew0;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->z, p1, j, k) = A3(curl->z, p1, j, k) - PW_G(s, (((p1 - 0.5) * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dx / c / mew0;
    }
    if (p2 >= 0 && p2 <= xe && sy != -1 && sz != -1) { /* :408-423 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl->y, p2, j, k) = A3(curl->y, p2, j, k) - PW_G(s, (((p2 + 0.5) * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dx / c / mew0;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->z, p2, j, k) = A3(curl->z, p2, j, k) + PW_G(s, (((p2 + 0.5) * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dx / c / mew0;
    }
    if (q1 >= 0 && q1 <= ye && sx != -1 && sz != -1) { /* :427-442 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl->x, i, q1, k) = A3(curl->x, i, q1, k) - PW_G(s, (((i + 0.5) * dx * kx + (q1 - 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dy / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->z, i, q1, k) = A3(curl->z, i, q1, k) + PW_G(s, ((i * dx * kx + (q1 - 0.5) * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dy / c / mew0;
    }
    if (q2 >= 0 && q2 <= ye && sx != -1 && sz != -1) { /* :443-458 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl->x, i, q2, k) = A3(curl->x, i, q2, k) + PW_G(s, (((i + 0.5) * dx * kx + (q2 + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dy / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl->z, i, q2, k) = A3(curl->z, i, q2, k) - PW_G(s, ((i * dx * kx + (q2 + 0.5) * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dy / c / mew0;
    }
    if (r1 >= 0 && r1 <= ze && sx != -1 && sy != -1) { /* :463-478 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl->x, i, j, r1) = A3(curl->x, i, j, r1) + PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + (r1 - 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dz / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl->y, i, j, r1) = A3(curl->y, i, j, r1) - PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + (r1 - 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dz / c / mew0;
    }
    if (r2 >= 0 && r2 <= ze && sx != -1 && sy != -1) { /* :479-494 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl->x, i, j, r2) = A3(curl->x, i, j, r2) - PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + (r2 + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dz / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl->y, i, j, r2) = A3(curl->y, i, j, r2) + PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + (r2 + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dz / c / mew0;
    }
  }
}

/* maxwell::plane_wave_execute(vfield*,vfield*,int) maxwell.cc:512-812 (PML drivers) */
static void plane_wave_execute_adv(ox_sim* s, vf* curl1, vf* curl2, int timestep) {
  double dx = s->dx, dy = s->dy, dz = s->dz, kx = s->kx, ky = s->ky, kz = s->kz, init = s->init, c = s->c, mew0 = s->mew0;
  int p1 = s->p1, p2 = s->p2, q1 = s->q1, q2 = s->q2, r1 = s->r1, r2 = s->r2;
  int sx = s->start_x, ex = s->end_x, sy = s->start_y, ey = s->end_y, sz = s->start_z, ez = s->end_z;
  int xe = s->Nx - 1, ye = s->planar ? 0 : s->Ny - 1, ze = s->Nz - 1;
  double tm = timestep - 0.5, tp = timestep;
  if (s->planar) {
    if (curl1->face) {
      if ((p1 - 1) >= 0 && (p1 - 1) <= xe && sz != -1) /* :519-526 */
        for (int k = sz; k <= ez; k++)
          A3(curl1->z, p1 - 1, 0, k) = A3(curl1->z, p1 - 1, 0, k) + PW_G(s, ((p1 * dx * kx + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      if (p2 >= 0 && p2 <= xe && sz != -1) /* :527-534 */
        for (int k = sz; k <= ez; k++)
          A3(curl1->z, p2, 0, k) = A3(curl1->z, p2, 0, k) - PW_G(s, ((p2 * dx * kx + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      if ((r1 - 1) >= 0 && (r1 - 1) <= ze && sx != -1) /* :539-546 */
        for (int i = sx; i <= ex; i++)
          A3(curl2->x, i, 0, r1 - 1) = A3(curl2->x, i, 0, r1 - 1) + PW_G(s, ((i * dx * kx + r1 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
      if (r2 >= 0 && r2 <= ze && sx != -1) /* :547-553 */
        for (int i = sx; i <= ex; i++)
          A3(curl2->x, i, 0, r2) = A3(curl2->x, i, 0, r2) - PW_G(s, ((i * dx * kx + r2 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
    } else {
      if (p1 >= 0 && p1 <= xe && sz != -1) /* :559-565 */
        for (int k = sz; k <= ez; k++)
          A3(curl2->y, p1, 0, k) = A3(curl2->y, p1, 0, k) - PW_G(s, (((p1 - 0.5) * dx * kx + k * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_z_dir / dx / c / mew0;
      if (p2 >= 0 && p2 <= xe && sz != -1) /* :566-572 */
        for (int k = sz; k <= ez; k++)
          A3(curl2->y, p2, 0, k) = A3(curl2->y, p2, 0, k) + PW_G(s, (((p2 + 0.5) * dx * kx + k * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_z_dir / dx / c / mew0;
      if (r1 >= 0 && r1 <= ze && sx != -1) /* :577-583 */
        for (int i = sx; i <= ex; i++)
          A3(curl1->y, i, 0, r1) = A3(curl1->y, i, 0, r1) - PW_G(s, ((i * dx * kx + (r1 - 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_x_dir / dz / c / mew0;
      if (r2 >= 0 && r2 <= ze && sx != -1) /* :584-590 */
        for (int i = sx; i <= ex; i++)
          A3(curl1->y, i, 0, r2) = A3(curl1->y, i, 0, r2) + PW_G(s, ((i * dx * kx + (r2 + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * (-1) * s->H_x_dir / dz / c / mew0;
    }
    return;
  }
  if (curl1->face) {
    if ((p1 - 1) >= 0 && (p1 - 1) <= xe && sy != -1 && sz != -1) { /* :599-614 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl1->z, p1 - 1, j, k) = A3(curl1->z, p1 - 1, j, k) - PW_G(s, ((p1 * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl2->y, p1 - 1, j, k) = A3(curl2->y, p1 - 1, j, k) - PW_G(s, ((p1 * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dx;
    }
    if (p2 >= 0 && p2 <= xe && sy != -1 && sz != -1) { /* :615-630 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl1->z, p2, j, k) = A3(curl1->z, p2, j, k) + PW_G(s, ((p2 * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dx;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl2->y, p2, j, k) = A3(curl2->y, p2, j, k) + PW_G(s, ((p2 * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dx;
    }
    if ((q1 - 1) >= 0 && (q1 - 1) <= ye && sx != -1 && sz != -1) { /* :634-649 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl2->z, i, q1 - 1, k) = A3(curl2->z, i, q1 - 1, k) - PW_G(s, (((i + 0.5) * dx * kx + q1 * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dy;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl1->x, i, q1 - 1, k) = A3(curl1->x, i, q1 - 1, k) - PW_G(s, ((i * dx * kx + q1 * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dy;
    }
    if (q2 >= 0 && q2 <= ye && sx != -1 && sz != -1) { /* :650-665 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl2->z, i, q2, k) = A3(curl2->z, i, q2, k) + PW_G(s, (((i + 0.5) * dx * kx + q2 * dy * ky + k * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dy;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl1->x, i, q2, k) = A3(curl1->x, i, q2, k) + PW_G(s, ((i * dx * kx + q2 * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tm))) * s->E_z_dir / dy;
    }
    if ((r1 - 1) >= 0 && (r1 - 1) <= ze && sx != -1 && sy != -1) { /* :670-685 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl1->y, i, j, r1 - 1) = A3(curl1->y, i, j, r1 - 1) - PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + r1 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dz;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl2->x, i, j, r1 - 1) = A3(curl2->x, i, j, r1 - 1) - PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + r1 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
    }
    if (r2 >= 0 && r2 <= ze && sx != -1 && sy != -1) { /* :686-701 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl1->y, i, j, r2) = A3(curl1->y, i, j, r2) + PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + r2 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_x_dir / dz;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl2->x, i, j, r2) = A3(curl2->x, i, j, r2) + PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + r2 * dz * kz) + init * dx - PW_T(s, tm))) * s->E_y_dir / dz;
    }
  } else {
    if (p1 >= 0 && p1 <= xe && sy != -1 && sz != -1) { /* :707-722 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl2->y, p1, j, k) = A3(curl2->y, p1, j, k) - PW_G(s, (((p1 - 0.5) * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dx / c / mew0;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl1->z, p1, j, k) = A3(curl1->z, p1, j, k) - PW_G(s, (((p1 - 0.5) * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dx / c / mew0;
    }
    if (p2 >= 0 && p2 <= xe && sy != -1 && sz != -1) { /* :723-738 */
      for (int j = sy; j <= ey - 1; j++)
        for (int k = sz; k <= ez; k++)
          A3(curl2->y, p2, j, k) = A3(curl2->y, p2, j, k) + PW_G(s, (((p2 + 0.5) * dx * kx + (j + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dx / c / mew0;
      for (int j = sy; j <= ey; j++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl1->z, p2, j, k) = A3(curl1->z, p2, j, k) + PW_G(s, (((p2 + 0.5) * dx * kx + j * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dx / c / mew0;
    }
    if (q1 >= 0 && q1 <= ye && sx != -1 && sz != -1) { /* :742-757 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl1->x, i, q1, k) = A3(curl1->x, i, q1, k) - PW_G(s, (((i + 0.5) * dx * kx + (q1 - 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dy / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl2->z, i, q1, k) = A3(curl2->z, i, q1, k) - PW_G(s, ((i * dx * kx + (q1 - 0.5) * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dy / c / mew0;
    }
    if (q2 >= 0 && q2 <= ye && sx != -1 && sz != -1) { /* :758-773 */
      for (int i = sx; i <= ex - 1; i++)
        for (int k = sz; k <= ez; k++)
          A3(curl1->x, i, q2, k) = A3(curl1->x, i, q2, k) + PW_G(s, (((i + 0.5) * dx * kx + (q2 + 0.5) * dy * ky + k * dz * kz) + init * dx - PW_T(s, tp))) * s->H_z_dir / dy / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int k = sz; k <= ez - 1; k++)
          A3(curl2->z, i, q2, k) = A3(curl2->z, i, q2, k) + PW_G(s, ((i * dx * kx + (q2 + 0.5) * dy * ky + (k + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dy / c / mew0;
    }
    if (r1 >= 0 && r1 <= ze && sx != -1 && sy != -1) { /* :778-793 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl2->x, i, j, r1) = A3(curl2->x, i, j, r1) - PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + (r1 - 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dz / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl1->y, i, j, r1) = A3(curl1->y, i, j, r1) - PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + (r1 - 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dz / c / mew0;
    }
    if (r2 >= 0 && r2 <= ze && sx != -1 && sy != -1) { /* :794-809 */
      for (int i = sx; i <= ex - 1; i++)
        for (int j = sy; j <= ey; j++)
          A3(curl2->x, i, j, r2) = A3(curl2->x, i, j, r2) + PW_G(s, (((i + 0.5) * dx * kx + j * dy * ky + (r2 + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_y_dir / dz / c / mew0;
      for (int i = sx; i <= ex; i++)
        for (int j = sy; j <= ey - 1; j++)
          A3(curl1->y, i, j, r2) = A3(curl1->y, i, j, r2) + PW_G(s, ((i * dx * kx + (j + 0.5) * dy * ky + (r2 + 0.5) * dz * kz) + init * dx - PW_T(s, tp))) * s->H_x_dir / dz / c / mew0;
    }
  }
}

/* ------------------------------------------------------------------ drivers */

/* Point source at the start of a step.  Reference: hard CW on E->Vz
 * (three_dim.cc:85-89, three_dim_pml.cc:161-165) with check_global_limits maxwell.cc:944-959
 * (x in [0,Nx-1], y in [0,Ny-1]; z unchecked).  Extension: additive Gaussian pulse. */
static void point_source(ox_sim* s, int t) {
  if (!s->p.usePS) return;
  int x = s->p.Nx_source, y = s->p.Ny_source, z = s->p.Nz_source;
  if (s->planar) y = 0;
  if (!(x >= 0 && y >= 0 && x <= s->Nx - 1 && y <= (s->planar ? 0 : s->Ny - 1))) return;
  if (s->p.source_kind == LX_SRC_CW_HARD) {
    /* int * int product first, as amp_source*sin(omega_source*t*dt) with int members */
    int wt = (int)((unsigned)s->omega_source * (unsigned)t);
    A3(s->E.z, x, y, z) = s->amp_source * sin(wt * s->dt);
  } else {
    double u = (t - s->p.src_t0) / s->p.src_tw;
    double v = s->p.amp_source * exp(-(u * u)) * sin(s->p.omega_source * t * s->dt);
    if (s->planar) A3(s->E.y, x, 0, z) = A3(s->E.y, x, 0, z) + v;
    else A3(s->E.z, x, y, z) = A3(s->E.z, x, y, z) + v;
  }
}

static double max_sq(const arr3* f, int nt) {
  size_t n = (size_t)f->n0 * f->n1 * f->n2;
  double m = -1.0;
  int first = 1;
  /* blitz::max(F*F) (two_dim_pml.cc:181): serial reduction order does not change a max */
  (void)nt;
  for (size_t q = 0; q < n; q++) {
    double v = f->a[q] * f->a[q];
    if (first || v > m) { m = v; first = 0; }
  }
  return n ? m : 0.0;
}

/* Etotal = |E|^2 over (Nx-1,Ny-1,Nz-1) into the Ez-shaped array, then its max
 * (three_dim.cc:180-189, three_dim_pml.cc:266-276). */
static void etotal_3d(ox_sim* s) {
  int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz, nt = s->threads;
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < (Ny - 1); j++)
      for (int k = 0; k < (Nz - 1); k++)
        A3(s->Etotal, i, j, k) = A3(s->E.z, i, j, k) * A3(s->E.z, i, j, k) + A3(s->E.y, i, j, k) * A3(s->E.y, i, j, k) + A3(s->E.x, i, j, k) * A3(s->E.x, i, j, k);
  size_t n = (size_t)s->Etotal.n0 * s->Etotal.n1 * s->Etotal.n2;
  double m = s->Etotal.a[0];
  for (size_t q = 1; q < n; q++)
    if (s->Etotal.a[q] > m) m = s->Etotal.a[q];
  s->local_max = m;
}

static void record_probes(ox_sim* s) {
  if (s->nprobes <= 0 || s->probe_rows >= s->probe_cap) return;
  double* row = s->probe_buf + (size_t)s->probe_rows * s->nprobes * 6;
  for (int q = 0; q < s->nprobes; q++) {
    int i = s->probe_ijk[3 * q], j = s->probe_ijk[3 * q + 1], k = s->probe_ijk[3 * q + 2];
    for (int c = 0; c < 6; c++) {
      arr3* f = comp_arr(s, c);
      int sh[3];
      ox_field_shape(s, c, sh);
      double v = 0.0;
      if (i >= 0 && j >= 0 && k >= 0 && i < sh[0] && j < sh[1] && k < sh[2]) v = A3(*f, i, j, k);
      row[q * 6 + c] = v;
    }
  }
  s->probe_rows++;
}

int ox_add_dft_plane(ox_sim* s, int axis, int index, int nfreq, const double* omega, int every) {
  static const int comps[3][4] = {{LX_EY, LX_EZ, LX_HY, LX_HZ}, {LX_EZ, LX_EX, LX_HZ, LX_HX}, {LX_EX, LX_EY, LX_HX, LX_HY}};
  if (s->ndft >= OX_MAX_DFT || axis < 0 || axis > 2 || (s->planar && axis == 1) || nfreq < 1 || every < 1) return -1;
  int N[3] = {s->Nx, s->Ny, s->Nz};
  if (index < 0 || index >= N[axis]) return -1;
  ox_dft* d = &s->dft[s->ndft];
  d->axis = axis; d->index = index; d->nfreq = nfreq; d->every = every;
  d->na = axis == 0 ? s->Ny : s->Nx;
  d->nb = axis == 2 ? s->Ny : s->Nz;
  for (int q = 0; q < 4; q++) d->comp[q] = comps[axis][q];
  d->omega = (double*)malloc(sizeof(double) * (size_t)nfreq);
  d->acc = (double*)calloc((size_t)nfreq * 4 * d->na * d->nb * 2, sizeof(double));
  if (!d->omega || !d->acc) return -1;
  memcpy(d->omega, omega, sizeof(double) * (size_t)nfreq);
  return s->ndft++;
}

int ox_read_dft(ox_sim* s, int id, double* out, size_t n) {
  if (id < 0 || id >= s->ndft) return LX_ERR_INVALID;
  ox_dft* d = &s->dft[id];
  size_t m = (size_t)d->nfreq * 4 * d->na * d->nb * 2;
  if (n != m) return LX_ERR_INVALID;
  memcpy(out, d->acc, m * sizeof(double));
  return LX_OK;
}

/* acc += every * F(t+1) e^{-i w (t+1) dt} for E, every * F(t+1/2) e^{-i w (t+1/2) dt} for H */
static void record_dft(ox_sim* s, int t) {
  for (int q = 0; q < s->ndft; q++) {
    ox_dft* d = &s->dft[q];
    if (t % d->every != 0) continue;
    size_t nc = (size_t)d->na * d->nb;
    for (int comp = 0; comp < 4; comp++) {
      arr3* f = comp_arr(s, d->comp[comp]);
      int sh[3];
      ox_field_shape(s, d->comp[comp], sh);
      for (int fq = 0; fq < d->nfreq; fq++) {
        double ph = comp < 2 ? d->omega[fq] * ((double)(t + 1) * s->dt) : d->omega[fq] * (((double)t + 0.5) * s->dt);
        double c = cos(ph), sn = sin(ph);
        double* acc = d->acc + ((size_t)fq * 4 + comp) * nc * 2;
        for (int a = 0; a < d->na; a++)
          for (int b = 0; b < d->nb; b++) {
            int u[3];
            u[d->axis] = d->index;
            u[d->axis == 0 ? 1 : 0] = a;
            u[d->axis == 2 ? 1 : 2] = b;
            double v = 0.0;
            if (u[0] < sh[0] && u[1] < sh[1] && u[2] < sh[2]) v = A3(*f, u[0], u[1], u[2]);
            v = v * (double)d->every;
            size_t cell = (size_t)a * d->nb + b;
            acc[2 * cell] = fma(v, c, acc[2 * cell]);
            acc[2 * cell + 1] = fma(-v, sn, acc[2 * cell + 1]);
          }
      }
    }
  }
}

/* maxwell::solve_planar two_dim.cc:85-144 (one iteration) */
static void step_planar(ox_sim* s, int t) {
  int Nx = s->Nx, Nz = s->Nz, nt = s->threads;
  double Ca = 1.0, Da = 1.0, Db = s->dt / s->mew0; /* :52-53 */
  point_source(s, t);
  curl_planar(s, &s->E, &s->Ecurl); /* :95 */
  if (s->p.usePW) plane_wave_execute(s, &s->Ecurl, t);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < (Nz - 1); j++)
      A3(s->H.x, i, 0, j) = Da * A3(s->H.x, i, 0, j) - Db * A3(s->Ecurl.x, i, 0, j); /* :103 */
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < Nz; j++)
      A3(s->H.z, i, 0, j) = Da * A3(s->H.z, i, 0, j) - Db * A3(s->Ecurl.z, i, 0, j); /* :109 */
  curl_planar(s, &s->H, &s->Hcurl); /* :113 */
  if (s->p.usePW) plane_wave_execute(s, &s->Hcurl, t);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < (Nz - 1); j++)
      A3(s->E.y, i, 0, j) = Ca * A3(s->E.y, i, 0, j) + A3(s->Cb.y, i, 0, j) * A3(s->Hcurl.y, i, 0, j); /* :121 */
  s->local_max = max_sq(&s->E.y, nt); /* :128 */
}

/* maxwell::solve_planar_pml two_dim_pml.cc:126-188 (one iteration) */
static void step_planar_pml(ox_sim* s, int t) {
  int Nx = s->Nx, Nz = s->Nz, nt = s->threads;
  double Ca = 1.0, Da = 1.0, Dbv = s->dt / s->mew0; /* :55, Db arrays = dt/mew0 :117-118 */
  const double *b_hz = s->b_h[2], *c_hz = s->c_h[2], *k_hz = s->k_h[2];
  const double *b_hx = s->b_h[0], *c_hx = s->c_h[0], *k_hx = s->k_h[0];
  const double *b_ez = s->b_e[2], *c_ez = s->c_e[2], *k_ez = s->k_e[2];
  const double *b_ex = s->b_e[0], *c_ex = s->c_e[0], *k_ex = s->k_e[0];
  point_source(s, t);
  curl_planar_adv(s, &s->E, &s->Ecurl1, &s->Ecurl2); /* :144 */
  if (s->p.usePW) plane_wave_execute_adv(s, &s->Ecurl1, &s->Ecurl2, t);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < (Nz - 1); j++) { /* :149-155 */
      A3(s->psi_H2.x, i, 0, j) = b_hz[j] * A3(s->psi_H2.x, i, 0, j) + c_hz[j] * A3(s->Ecurl2.x, i, 0, j);
      A3(s->H.x, i, 0, j) = Da * A3(s->H.x, i, 0, j) - Dbv * (-A3(s->Ecurl2.x, i, 0, j) / k_hz[j] - A3(s->psi_H2.x, i, 0, j));
    }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < Nz; j++) { /* :156-162 */
      A3(s->psi_H1.z, i, 0, j) = b_hx[i] * A3(s->psi_H1.z, i, 0, j) + c_hx[i] * A3(s->Ecurl1.z, i, 0, j);
      A3(s->H.z, i, 0, j) = Da * A3(s->H.z, i, 0, j) - Dbv * (A3(s->Ecurl1.z, i, 0, j) / k_hx[i] + A3(s->psi_H1.z, i, 0, j));
    }
  curl_planar_adv(s, &s->H, &s->Hcurl1, &s->Hcurl2); /* :164 */
  if (s->p.usePW) plane_wave_execute_adv(s, &s->Hcurl1, &s->Hcurl2, t);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < (Nz - 1); j++) { /* :169-176 */
      A3(s->psi_E1.y, i, 0, j) = b_ez[j] * A3(s->psi_E1.y, i, 0, j) + c_ez[j] * A3(s->Hcurl1.y, i, 0, j);
      A3(s->psi_E2.y, i, 0, j) = b_ex[i] * A3(s->psi_E2.y, i, 0, j) + c_ex[i] * A3(s->Hcurl2.y, i, 0, j);
      A3(s->E.y, i, 0, j) = Ca * A3(s->E.y, i, 0, j) + A3(s->Cb.y, i, 0, j) * (A3(s->Hcurl1.y, i, 0, j) / k_ez[j] - A3(s->Hcurl2.y, i, 0, j) / k_ex[i] + A3(s->psi_E1.y, i, 0, j) - A3(s->psi_E2.y, i, 0, j));
    }
  s->local_max = max_sq(&s->E.y, nt); /* :181 */
}

/* maxwell::solve3d three_dim.cc:82-196 (one iteration) */
static void step_3d(ox_sim* s, int t) {
  int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz, nt = s->threads;
  double Ca = 1.0, Da = 1.0, Db = s->dt / s->mew0; /* :53-55 */
  point_source(s, t);
  curl_3d(s, &s->E, &s->Ecurl); /* :101 */
  if (s->p.usePW) plane_wave_execute(s, &s->Ecurl, t);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < (Ny - 1); j++)
      for (int k = 0; k < (Nz - 1); k++)
        A3(s->H.x, i, j, k) = Da * A3(s->H.x, i, j, k) - Db * A3(s->Ecurl.x, i, j, k); /* :111 */
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < Ny; j++)
      for (int k = 0; k < (Nz - 1); k++)
        A3(s->H.y, i, j, k) = Da * A3(s->H.y, i, j, k) - Db * A3(s->Ecurl.y, i, j, k); /* :120 */
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < (Ny - 1); j++)
      for (int k = 0; k < Nz; k++)
        A3(s->H.z, i, j, k) = Da * A3(s->H.z, i, j, k) - Db * A3(s->Ecurl.z, i, j, k); /* :129 */
  curl_3d(s, &s->H, &s->Hcurl); /* :134 */
  if (s->p.usePW) plane_wave_execute(s, &s->Hcurl, t);
  /* Cb is the scalar dt/epsilon0 in the reference (:54); the restatement reads the Cb
   * arrays, which hold that value unless a material was set (extension). */
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < Ny; j++)
      for (int k = 0; k < Nz; k++)
        A3(s->E.x, i, j, k) = Ca * A3(s->E.x, i, j, k) + A3(s->Cb.x, i, j, k) * A3(s->Hcurl.x, i, j, k); /* :144 */
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < (Ny - 1); j++)
      for (int k = 0; k < Nz; k++)
        A3(s->E.y, i, j, k) = Ca * A3(s->E.y, i, j, k) + A3(s->Cb.y, i, j, k) * A3(s->Hcurl.y, i, j, k); /* :153 */
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < Ny; j++)
      for (int k = 0; k < (Nz - 1); k++)
        A3(s->E.z, i, j, k) = Ca * A3(s->E.z, i, j, k) + A3(s->Cb.z, i, j, k) * A3(s->Hcurl.z, i, j, k); /* :162 */
  etotal_3d(s); /* :180-189 */
}

/* maxwell::solve3d_pml three_dim_pml.cc:158-283 (one iteration) */
static void step_3d_pml(ox_sim* s, int t) {
  int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz, nt = s->threads;
  double Ca = 1.0, Da = 1.0, Db = s->dt / s->mew0; /* :53, Db arrays = dt/mew0 :130-132 */
  const double *k_ex = s->k_e[0], *k_ey = s->k_e[1], *k_ez = s->k_e[2];
  const double *k_hx = s->k_h[0], *k_hy = s->k_h[1], *k_hz = s->k_h[2];
  const double *b_ex = s->b_e[0], *b_ey = s->b_e[1], *b_ez = s->b_e[2];
  const double *b_hx = s->b_h[0], *b_hy = s->b_h[1], *b_hz = s->b_h[2];
  const double *c_ex = s->c_e[0], *c_ey = s->c_e[1], *c_ez = s->c_e[2];
  const double *c_hx = s->c_h[0], *c_hy = s->c_h[1], *c_hz = s->c_h[2];
  vf *E = &s->E, *H = &s->H, *Cb = &s->Cb;
  vf *Ecurl1 = &s->Ecurl1, *Ecurl2 = &s->Ecurl2, *Hcurl1 = &s->Hcurl1, *Hcurl2 = &s->Hcurl2;
  vf *psi_E1 = &s->psi_E1, *psi_E2 = &s->psi_E2, *psi_H1 = &s->psi_H1, *psi_H2 = &s->psi_H2;
  point_source(s, t);
  curl_3d_adv(s, E, Ecurl1, Ecurl2); /* :176 */
  if (s->p.usePW) plane_wave_execute_adv(s, Ecurl1, Ecurl2, t);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < (Ny - 1); j++)
      for (int k = 0; k < (Nz - 1); k++) { /* :182-191 */
        A3(psi_H1->x, i, j, k) = b_hy[j] * A3(psi_H1->x, i, j, k) + c_hy[j] * A3(Ecurl1->x, i, j, k);
        A3(psi_H2->x, i, j, k) = b_hz[k] * A3(psi_H2->x, i, j, k) + c_hz[k] * A3(Ecurl2->x, i, j, k);
        A3(H->x, i, j, k) = Da * A3(H->x, i, j, k) - Db * (A3(Ecurl1->x, i, j, k) / k_hy[j] - A3(Ecurl2->x, i, j, k) / k_hz[k]) - Db * (A3(psi_H1->x, i, j, k) - A3(psi_H2->x, i, j, k));
      }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < Ny; j++)
      for (int k = 0; k < (Nz - 1); k++) { /* :193-202 */
        A3(psi_H1->y, i, j, k) = b_hz[k] * A3(psi_H1->y, i, j, k) + c_hz[k] * A3(Ecurl1->y, i, j, k);
        A3(psi_H2->y, i, j, k) = b_hx[i] * A3(psi_H2->y, i, j, k) + c_hx[i] * A3(Ecurl2->y, i, j, k);
        A3(H->y, i, j, k) = Da * A3(H->y, i, j, k) - Db * (A3(Ecurl1->y, i, j, k) / k_hz[k] - A3(Ecurl2->y, i, j, k) / k_hx[i]) - Db * (A3(psi_H1->y, i, j, k) - A3(psi_H2->y, i, j, k));
      }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < (Ny - 1); j++)
      for (int k = 0; k < Nz; k++) { /* :204-213 */
        A3(psi_H1->z, i, j, k) = b_hx[i] * A3(psi_H1->z, i, j, k) + c_hx[i] * A3(Ecurl1->z, i, j, k);
        A3(psi_H2->z, i, j, k) = b_hy[j] * A3(psi_H2->z, i, j, k) + c_hy[j] * A3(Ecurl2->z, i, j, k);
        A3(H->z, i, j, k) = Da * A3(H->z, i, j, k) - Db * (A3(Ecurl1->z, i, j, k) / k_hx[i] - A3(Ecurl2->z, i, j, k) / k_hy[j]) - Db * (A3(psi_H1->z, i, j, k) - A3(psi_H2->z, i, j, k));
      }
  curl_3d_adv(s, H, Hcurl1, Hcurl2); /* :218 */
  if (s->p.usePW) plane_wave_execute_adv(s, Hcurl1, Hcurl2, t);
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < (Nx - 1); i++)
    for (int j = 0; j < Ny; j++)
      for (int k = 0; k < Nz; k++) { /* :224-233 */
        A3(psi_E1->x, i, j, k) = b_ey[j] * A3(psi_E1->x, i, j, k) + c_ey[j] * A3(Hcurl1->x, i, j, k);
        A3(psi_E2->x, i, j, k) = b_ez[k] * A3(psi_E2->x, i, j, k) + c_ez[k] * A3(Hcurl2->x, i, j, k);
        A3(E->x, i, j, k) = Ca * A3(E->x, i, j, k) + A3(Cb->x, i, j, k) * (A3(Hcurl1->x, i, j, k) / k_ey[j] - A3(Hcurl2->x, i, j, k) / k_ez[k]) + A3(Cb->x, i, j, k) * (A3(psi_E1->x, i, j, k) - A3(psi_E2->x, i, j, k));
      }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < (Ny - 1); j++)
      for (int k = 0; k < Nz; k++) { /* :235-244 */
        A3(psi_E1->y, i, j, k) = b_ez[k] * A3(psi_E1->y, i, j, k) + c_ez[k] * A3(Hcurl1->y, i, j, k);
        A3(psi_E2->y, i, j, k) = b_ex[i] * A3(psi_E2->y, i, j, k) + c_ex[i] * A3(Hcurl2->y, i, j, k);
        A3(E->y, i, j, k) = Ca * A3(E->y, i, j, k) + A3(Cb->y, i, j, k) * (A3(Hcurl1->y, i, j, k) / k_ez[k] - A3(Hcurl2->y, i, j, k) / k_ex[i]) + A3(Cb->y, i, j, k) * (A3(psi_E1->y, i, j, k) - A3(psi_E2->y, i, j, k));
      }
#pragma omp parallel for num_threads(nt) schedule(dynamic)
  for (int i = 0; i < Nx; i++)
    for (int j = 0; j < Ny; j++)
      for (int k = 0; k < (Nz - 1); k++) { /* :246-255 */
        A3(psi_E1->z, i, j, k) = b_ex[i] * A3(psi_E1->z, i, j, k) + c_ex[i] * A3(Hcurl1->z, i, j, k);
        A3(psi_E2->z, i, j, k) = b_ey[j] * A3(psi_E2->z, i, j, k) + c_ey[j] * A3(Hcurl2->z, i, j, k);
        A3(E->z, i, j, k) = Ca * A3(E->z, i, j, k) + A3(Cb->z, i, j, k) * (A3(Hcurl1->z, i, j, k) / k_ex[i] - A3(Hcurl2->z, i, j, k) / k_ey[j]) + A3(Cb->z, i, j, k) * (A3(psi_E1->z, i, j, k) - A3(psi_E2->z, i, j, k));
      }
  etotal_3d(s); /* :266-276 */
}

/* maxwell::solve maxwell.cc:157-174 dispatch, one iteration per step. */
int ox_step(ox_sim* s, int nsteps) {
  for (int q = 0; q < nsteps; q++) {
    int t = s->t;
    if (s->planar) {
      if (s->pml) step_planar_pml(s, t);
      else step_planar(s, t);
    } else {
      if (s->pml) step_3d_pml(s, t);
      else step_3d(s, t);
    }
    s->t++;
    record_dft(s, t);
    record_probes(s);
  }
  return LX_OK;
}
