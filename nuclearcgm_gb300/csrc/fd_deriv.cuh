// First derivative along one lattice axis with the order-dropping stencils
// of Operators::derivative (src/operators/differential_operators.cpp:
// 482-543): two-point one-sided differences on the box faces, central
// differences of order 2, 4 and 6 on the next three layers, and the 9-point
// (order-8) central rule inside. g(q) returns the value at axis index q.
#pragma once

namespace ncgm {
namespace fd {

template <class T, class Get>
__device__ __forceinline__ T d1(const Get &g, int pos, int n, double h) {
  if (pos == 0) {
    return (g(pos + 1) - g(pos)) / h;
  } else if (pos == 1 || pos == n - 2) {
    return (g(pos + 1) - g(pos - 1)) / (2.0 * h);
  } else if (pos == n - 1) {
    return (g(pos) - g(pos - 1)) / h;
  } else if (pos == 2 || pos == n - 3) {
    T f_2 = g(pos - 2), f_1 = g(pos - 1), f1 = g(pos + 1), f2 = g(pos + 2);
    return (-f2 + 8.0 * f1 - 8.0 * f_1 + f_2) / (12.0 * h);
  } else if (pos == 3 || pos == n - 4) {
    T f_3 = g(pos - 3), f_2 = g(pos - 2), f_1 = g(pos - 1);
    T f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3);
    return (-f_3 + 9.0 * f_2 - 45.0 * f_1 + 45.0 * f1 - 9.0 * f2 + f3) /
           (60.0 * h);
  } else {
    T f_4 = g(pos - 4), f_3 = g(pos - 3), f_2 = g(pos - 2), f_1 = g(pos - 1);
    T f1 = g(pos + 1), f2 = g(pos + 2), f3 = g(pos + 3), f4 = g(pos + 4);
    return (3.0 * f_4 - 32.0 * f_3 + 168.0 * f_2 - 672.0 * f_1 + 672.0 * f1 -
            168.0 * f2 + 32.0 * f3 - 3.0 * f4) /
           (840.0 * h);
  }
}

} // namespace fd
} // namespace ncgm
