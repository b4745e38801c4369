// CPU oracle for the hybridgrains-gb300 test suite: common 2-vector / 2x2
// helpers.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product library links, loads or
// calls this code; the tests compare the CUDA path against it,
// and the CPU baseline that bench.py times beside the GPU numbers.
//
// The reference evaluates these operations through Eigen 3.3 fixed-size
// expressions. Eigen is not available here, so each helper spells out the
// scalar operations in the order a coefficient-wise Eigen evaluation performs
// them (left-to-right sums over the inner index, column-major storage). The
// file is compiled with -ffp-contract=off so that no multiply-add is fused.
// Parity with the real reference binary is unpinned: the reference cannot be
// built without Eigen, and it ships no golden vectors for this path.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

namespace hgo {

struct V2 {
  double x, y;
};

// 2x2 matrix, column-major like Eigen's Matrix22sc: a00 a10 a01 a11.
struct M2 {
  double a00, a10, a01, a11;
};

inline V2 add(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 sub(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 scl(double s, V2 a) { return {s * a.x, s * a.y}; }
inline double dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
inline double sqnorm(V2 a) { return a.x * a.x + a.y * a.y; }
inline double norm(V2 a) { return std::sqrt(sqnorm(a)); }
// Eigen 3.3 MatrixBase::normalized(): v / sqrt(squaredNorm()) when > 0.
inline V2 normalized(V2 a) {
  const double n2 = sqnorm(a);
  if (n2 > 0.0) {
    const double n = std::sqrt(n2);
    return {a.x / n, a.y / n};
  }
  return a;
}
// MathUtilities::cross for 2-vectors (scisim/Math/MathUtilities.h:21-23).
inline double cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }

inline M2 madd(M2 a, M2 b) {
  return {a.a00 + b.a00, a.a10 + b.a10, a.a01 + b.a01, a.a11 + b.a11};
}
inline M2 msub(M2 a, M2 b) {
  return {a.a00 - b.a00, a.a10 - b.a10, a.a01 - b.a01, a.a11 - b.a11};
}
inline M2 mscl(double s, M2 a) {
  return {s * a.a00, s * a.a10, s * a.a01, s * a.a11};
}
inline M2 mdiv(M2 a, double s) {
  return {a.a00 / s, a.a10 / s, a.a01 / s, a.a11 / s};
}
inline M2 mmul(M2 a, M2 b) {
  return {a.a00 * b.a00 + a.a01 * b.a10, a.a10 * b.a00 + a.a11 * b.a10,
          a.a00 * b.a01 + a.a01 * b.a11, a.a10 * b.a01 + a.a11 * b.a11};
}
inline M2 mT(M2 a) { return {a.a00, a.a01, a.a10, a.a11}; }
inline double mdet(M2 a) { return a.a00 * a.a11 - a.a10 * a.a01; }
inline double mtrace(M2 a) { return a.a00 + a.a11; }
// Frobenius norm, summed in storage order.
inline double mnorm(M2 a) {
  return std::sqrt(a.a00 * a.a00 + a.a10 * a.a10 + a.a01 * a.a01 +
                   a.a11 * a.a11);
}
inline M2 mident(double s) { return {s, 0.0, 0.0, s}; }
inline V2 mvec(M2 a, V2 v) {
  return {a.a00 * v.x + a.a01 * v.y, a.a10 * v.x + a.a11 * v.y};
}

} // namespace hgo
