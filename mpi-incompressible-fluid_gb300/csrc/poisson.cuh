// Host interface of the spectral Poisson solver (poisson.cu).
#pragma once

#include <functional>
#include <string>

#include "common.cuh"

namespace mifgpu {

// Plan of the 1-D transform along one axis: kind, FFT factorisation, line
// pairs per CTA, and device tables (twiddles in T, eigenvalues in double).
template <typename T>
struct AxisPlan {
  int kind = 0;  // 0 DCT-I (Neumann), 1 real DFT (periodic)
  int n = 0, L = 0;
  int nfac = 0;
  int fac[16] = {0};
  int P = 1, lg_lines = 1;
  // register-resident path (float): FFT length reg_L = reg_n1 * reg_n2 (a power
  // of two in 64..1024), 0 if unused. A DCT-I axis of n = N + 1 points runs as
  // one length-N transform per line pair (reg_half, kernel kind 2); a periodic
  // axis as its length-n real DFT.
  int reg_n1 = 0, reg_n2 = 0, reg_P = 0, reg_lg = 0, reg_L = 0;
  bool reg_half = false;
  size_t reg_smem = 0;
  typename Vec2<T>::type *reg_tw = nullptr;  // exp(-2 pi i e / reg_L)
  typename Vec2<T>::type *dsc = nullptr;     // (sin, cos)(pi j / N), j < N (reg_half)
  bool pow2 = false;
  bool line_fast = false;
  size_t smem = 0;
  typename Vec2<T>::type *tw = nullptr;
  double *lam_dev = nullptr;

  int build(int kind, int n, double h, int line_count, bool line_fast, std::string &err);
  void release();
};

template <typename T>
struct PoissonSolver {
  Geometry geo{};
  AxisPlan<T> axis[3];
  T *eig = nullptr;  // 1/(lambda sum) on the owner block, x fastest; 0 at the zero mode
  int *err_flag = nullptr;  // device: set to 1 if a line kernel gave up waiting for its TMA loads

  int init(const Geometry &g, std::string &err);
  void release();
  // In place on the owner block of phi: rhs in, solution out (no periodic refresh).
  // `mark`, when set, is called with the sweep id (0 x-forward, 1 y-forward,
  // 2 z forward+eigen+inverse, 3 y-inverse, 4 x-inverse) before each launch.
  int solve(T *phi, cudaStream_t stream, long long *launches, const std::function<void(int)> &mark = nullptr);
};

}  // namespace mifgpu
