// Compile-time Butcher tableaux of the reference's embedded Runge-Kutta pairs.
//
// Coefficients are the same IEEE quotients the reference computes at run time
// (src/ivp/rk.rs:435-525 for RKF45, :568-620 for Bogacki-Shampine 3(2)).
// M(i, j) is the matrix entry the reference's stage loop reads for stage i
// and stage value j (rk.rs:370-374):
//   as_compiled  nalgebra from_vec fills column-major (rk.rs:459, :580), so
//                row_iter row i holds column i of the literal;
//   as_written   the literal read row by row;
//   fehlberg     as_written with 1859/4014 (rk.rs:499) replaced by 1859/4104.
// Zero entries are skipped at compile time by the kernels; the reference adds
// 0 * K_j, which only matters when K_j is not finite, and the kernels
// reproduce that case with a non-finite mask.
#pragma once

namespace bacon {

enum Layout : int { kAsCompiled = 0, kAsWritten = 1, kFehlberg = 2 };

struct Rkf45Literal {
  static constexpr int S = 6;
  // Written (row-major) matrix; entry [5][3] depends on the variant.
  __host__ __device__ static constexpr double a(int i, int j, bool fehlberg) {
    return (i == 1 && j == 0)   ? 1.0 / 4.0
           : (i == 2 && j == 0) ? 3.0 / 32.0
           : (i == 2 && j == 1) ? 9.0 / 32.0
           : (i == 3 && j == 0) ? 1932.0 / 2197.0
           : (i == 3 && j == 1) ? -7200.0 / 2197.0
           : (i == 3 && j == 2) ? 7296.0 / 2197.0
           : (i == 4 && j == 0) ? 439.0 / 216.0
           : (i == 4 && j == 1) ? -8.0
           : (i == 4 && j == 2) ? 3680.0 / 513.0
           : (i == 4 && j == 3) ? -845.0 / 4104.0
           : (i == 5 && j == 0) ? -8.0 / 27.0
           : (i == 5 && j == 1) ? 2.0
           : (i == 5 && j == 2) ? -3544.0 / 2565.0
           : (i == 5 && j == 3) ? (fehlberg ? 1859.0 / 4104.0 : 1859.0 / 4014.0)
           : (i == 5 && j == 4) ? -11.0 / 40.0
                                : 0.0;
  }
  __host__ __device__ static constexpr double c(int i) {
    return i == 0 ? 0.0 : i == 1 ? 1.0 / 4.0 : i == 2 ? 3.0 / 8.0 : i == 3 ? 12.0 / 13.0
           : i == 4 ? 1.0 : 1.0 / 2.0;
  }
  __host__ __device__ static constexpr double b(int i) {
    return i == 0 ? 25.0 / 216.0 : i == 1 ? 0.0 : i == 2 ? 1408.0 / 2565.0
           : i == 3 ? 2197.0 / 4104.0 : i == 4 ? -(1.0 / 5.0) : 0.0;
  }
  __host__ __device__ static constexpr double e(int i) {
    return i == 0 ? 1.0 / 360.0 : i == 1 ? 0.0 : i == 2 ? -128.0 / 4275.0
           : i == 3 ? -2197.0 / 75240.0 : i == 4 ? 1.0 / 50.0 : 2.0 / 55.0;
  }
};

struct Bs23Literal {
  static constexpr int S = 4;
  __host__ __device__ static constexpr double a(int i, int j, bool) {
    return (i == 1 && j == 0)   ? 1.0 / 2.0
           : (i == 2 && j == 1) ? 3.0 / 4.0
           : (i == 3 && j == 0) ? 2.0 / 9.0
           : (i == 3 && j == 1) ? 1.0 / 3.0
           : (i == 3 && j == 2) ? 4.0 / 9.0
                                : 0.0;
  }
  __host__ __device__ static constexpr double c(int i) {
    return i == 0 ? 0.0 : i == 1 ? 1.0 / 2.0 : i == 2 ? 3.0 / 4.0 : 1.0;
  }
  __host__ __device__ static constexpr double b(int i) {
    return i == 0 ? 2.0 / 9.0 : i == 1 ? 1.0 / 3.0 : i == 2 ? 4.0 / 9.0 : 0.0;
  }
  __host__ __device__ static constexpr double e(int i) {
    return i == 0 ? -5.0 / 72.0 : i == 1 ? 1.0 / 12.0 : i == 2 ? 1.0 / 9.0 : -(1.0 / 8.0);
  }
};

template <class Lit, int L>
struct Tableau {
  static constexpr int S = Lit::S;
  static constexpr int kLayout = L;
  __host__ __device__ static constexpr double M(int i, int j) {
    return L == kAsCompiled ? Lit::a(j, i, false) : Lit::a(i, j, L == kFehlberg);
  }
  __host__ __device__ static constexpr double c(int i) { return Lit::c(i); }
  __host__ __device__ static constexpr double b(int i) { return Lit::b(i); }
  __host__ __device__ static constexpr double e(int i) { return Lit::e(i); }
};

}  // namespace bacon
