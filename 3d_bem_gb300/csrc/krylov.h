// krylov.h -- device state and launch interface of the GMRES kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bemgpu {

struct GmresState {
  double bnorm;   // ||b||
  double beta;    // ||r|| at the last restart
  double resid;   // current relative residual estimate
  int jcount;     // Arnoldi steps taken in this cycle
  int iters;      // total steps
  int done;       // converged (or breakdown)
  int pad;
};

struct KrylovArgs {
  int64_t N;
  int R;
  int m;           // restart length
  double tol;
  double2* Vb;     // (m+1) x R x N basis
  double2* w;      // R x N work vector (operator output)
  double2* x;      // R x N solution
  double2* H;      // R x m x (m+1) Hessenberg columns
  double2* g;      // R x (m+1)
  double2* cs;     // R x m
  double2* sn;     // R x m
  double2* h;      // R x (m+1) projection coefficients
  double2* y;      // R x m
  double2* cpart;  // nct x R x (m+1) partial dots
  double* npart;   // nct x R partial norms
  double* hnorm;   // R
  GmresState* st;  // R
};

int krylov_num_ctas(int64_t N);
// one CGS2 Arnoldi step j on a.w; returns the kernels launched
int krylov_orthogonalize(const KrylovArgs& a, int j, cudaStream_t s);
void krylov_restart(const KrylovArgs& a, int init, cudaStream_t s);
void krylov_residual(const double2* b, double2* w, int64_t n, cudaStream_t s);
// partial[cta][r] = squared norm of v[r] over the CTA's chunk (krylov_num_ctas CTAs)
void krylov_norm_partials(const double2* v, int64_t N, int R, double* partial, cudaStream_t s);
// x[i] += d[i]
void krylov_axpy(double2* x, const double2* d, int64_t n, cudaStream_t s);
void krylov_update(const KrylovArgs& a, cudaStream_t s);

}  // namespace bemgpu
