// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// Operation-counting scalar for the algorithmic FP64 cost of the restated
// reference arithmetic. Instantiating the oracle's templates with Ops runs the
// reference's expressions as written and counts every floating-point
// operation whose operands include a state-dependent value (operations among
// mesh and basis constants alone are constants of the discretisation and are
// not counted). Convention: +, -, *, /, sqrt, |x| and max each count 1, so a
// multiply-add counts 2.
//
// The reverse (adjoint) cost is counted by the operation-by-operation rule of
// reverse-mode differentiation, which is what the reference's Enzyme call
// performs on the same code: each operation's adjoint statement costs
//   c = a +- b      a_bar += c_bar, b_bar +-= c_bar                 2 (1 with a constant operand)
//   c = a * b       a_bar += c_bar b, b_bar += c_bar a              4 (2 with a constant operand)
//   c = a / b       a_bar += c_bar / b, b_bar -= c_bar c / b        5 (2 if b is constant, 3 if a is)
//   c = sqrt(a)     a_bar += c_bar * 0.5 / c                        3
//   c = |a|, max    route c_bar to the chosen operand               1
// (the accumulation into an adjoint that is still zero is counted too).
#pragma once
#include <cmath>

#include "igr_common.hpp"

namespace igr {

struct OpTally {
  long long fwd = 0, rev = 0;
};
inline OpTally& op_tally() { static thread_local OpTally t; return t; }
inline void op_count(long long f, long long r) { op_tally().fwd += f; op_tally().rev += r; }

struct Ops {
  double v;
  Ops() : v(0.0) {}
  Ops(double x) : v(x) {}  // NOLINT (constants enter without cost)
};

inline Ops operator+(const Ops& a, const Ops& b) { op_count(1, 2); return Ops(a.v + b.v); }
inline Ops operator-(const Ops& a, const Ops& b) { op_count(1, 2); return Ops(a.v - b.v); }
inline Ops operator*(const Ops& a, const Ops& b) { op_count(1, 4); return Ops(a.v * b.v); }
inline Ops operator/(const Ops& a, const Ops& b) { op_count(1, 5); return Ops(a.v / b.v); }
inline Ops operator-(const Ops& a) { op_count(1, 1); return Ops(-a.v); }
inline Ops operator+(const Ops& a, double b) { op_count(1, 1); return Ops(a.v + b); }
inline Ops operator+(double a, const Ops& b) { op_count(1, 1); return Ops(a + b.v); }
inline Ops operator-(const Ops& a, double b) { op_count(1, 1); return Ops(a.v - b); }
inline Ops operator-(double a, const Ops& b) { op_count(1, 1); return Ops(a - b.v); }
inline Ops operator*(const Ops& a, double b) { op_count(1, 2); return Ops(a.v * b); }
inline Ops operator*(double a, const Ops& b) { op_count(1, 2); return Ops(a * b.v); }
inline Ops operator/(const Ops& a, double b) { op_count(1, 2); return Ops(a.v / b); }
inline Ops operator/(double a, const Ops& b) { op_count(1, 3); return Ops(a / b.v); }
inline Ops& operator+=(Ops& a, const Ops& b) { a = a + b; return a; }
inline Ops& operator-=(Ops& a, const Ops& b) { a = a - b; return a; }
inline Ops& operator*=(Ops& a, const Ops& b) { a = a * b; return a; }
inline bool operator<(const Ops& a, const Ops& b) { return a.v < b.v; }
inline bool operator>(const Ops& a, const Ops& b) { return a.v > b.v; }
inline bool operator>(const Ops& a, double b) { return a.v > b; }
inline bool operator<(const Ops& a, double b) { return a.v < b; }
inline Ops sqrt(const Ops& a) { op_count(1, 3); return Ops(std::sqrt(a.v)); }
inline Ops abs(const Ops& a) { op_count(1, 1); return Ops(std::fabs(a.v)); }
inline double value(const Ops& x) { return x.v; }
// max(a, b) (jmax): one comparison forward, one routed adjoint in reverse
inline Ops jmax(const Ops& a, const Ops& b) { op_count(1, 1); return (b.v > a.v) ? b : a; }

}  // namespace igr
