/*
 * flop_count.h -- TEST INFRASTRUCTURE ONLY: the counting scalar of the
 * op-counting build of the oracle (oracle/Makefile target
 * _ref/liboracle_count.so, made from vlct_oracle.cpp with every floating
 * type replaced by `oreal`).
 *
 * An oreal holds one double (same size and layout, so the oracle's block
 * structures keep their ABI) and counts every arithmetic operation done on
 * it: add/subtract, multiply, divide, square root, and -- not floating-point
 * operations, but counted apart -- comparisons, min/max and absolute values.
 * The values computed are the oracle's own (in double); only the counts are
 * new.
 */
#ifndef ORACLE_FLOP_COUNT_H
#define ORACLE_FLOP_COUNT_H
#include <cmath>

enum { OC_ADD = 0, OC_MUL, OC_DIV, OC_SQRT, OC_CMP, OC_MINMAX, OC_ABS, OC_N };
extern unsigned long long g_oracle_ops[OC_N];

struct oreal {
  double v;
  oreal() : v(0.0) {}
  oreal(double x) : v(x) {}
  oreal(float x) : v(x) {}
  oreal(int x) : v(x) {}
  oreal(long x) : v((double)x) {}
  oreal(unsigned x) : v(x) {}
  oreal(unsigned long x) : v((double)x) {}
  oreal(bool x) : v(x ? 1.0 : 0.0) {}
  explicit operator double() const { return v; }
  explicit operator int() const { return (int)v; }
  oreal& operator+=(oreal o) { g_oracle_ops[OC_ADD]++; v += o.v; return *this; }
  oreal& operator-=(oreal o) { g_oracle_ops[OC_ADD]++; v -= o.v; return *this; }
  oreal& operator*=(oreal o) { g_oracle_ops[OC_MUL]++; v *= o.v; return *this; }
  oreal& operator/=(oreal o) { g_oracle_ops[OC_DIV]++; v /= o.v; return *this; }
  oreal operator-() const { return oreal(-v); }
  oreal operator+() const { return *this; }
};

#define ORACLE_BIN(OP, K)                                                        \
  inline oreal operator OP(oreal a, oreal b) { g_oracle_ops[K]++; return oreal(a.v OP b.v); } \
  inline oreal operator OP(oreal a, double b) { g_oracle_ops[K]++; return oreal(a.v OP b); }  \
  inline oreal operator OP(double a, oreal b) { g_oracle_ops[K]++; return oreal(a OP b.v); }  \
  inline oreal operator OP(oreal a, int b) { g_oracle_ops[K]++; return oreal(a.v OP b); }     \
  inline oreal operator OP(int a, oreal b) { g_oracle_ops[K]++; return oreal(a OP b.v); }
ORACLE_BIN(+, OC_ADD)
ORACLE_BIN(-, OC_ADD)
ORACLE_BIN(*, OC_MUL)
ORACLE_BIN(/, OC_DIV)
#undef ORACLE_BIN

#define ORACLE_CMP(OP)                                                           \
  inline bool operator OP(oreal a, oreal b) { g_oracle_ops[OC_CMP]++; return a.v OP b.v; } \
  inline bool operator OP(oreal a, double b) { g_oracle_ops[OC_CMP]++; return a.v OP b; }  \
  inline bool operator OP(double a, oreal b) { g_oracle_ops[OC_CMP]++; return a OP b.v; }  \
  inline bool operator OP(oreal a, int b) { g_oracle_ops[OC_CMP]++; return a.v OP b; }     \
  inline bool operator OP(int a, oreal b) { g_oracle_ops[OC_CMP]++; return a OP b.v; }
ORACLE_CMP(<)
ORACLE_CMP(>)
ORACLE_CMP(<=)
ORACLE_CMP(>=)
ORACLE_CMP(==)
ORACLE_CMP(!=)
#undef ORACLE_CMP

inline oreal osqrt(oreal a) { g_oracle_ops[OC_SQRT]++; return oreal(std::sqrt(a.v)); }
inline oreal ofabs(oreal a) { g_oracle_ops[OC_ABS]++; return oreal(std::fabs(a.v)); }
inline oreal ofmax(oreal a, oreal b) { g_oracle_ops[OC_MINMAX]++; return oreal(std::fmax(a.v, b.v)); }
inline oreal ofmin(oreal a, oreal b) { g_oracle_ops[OC_MINMAX]++; return oreal(std::fmin(a.v, b.v)); }
inline oreal omax(oreal a, oreal b) { g_oracle_ops[OC_MINMAX]++; return (a.v < b.v) ? b : a; }
inline oreal omin(oreal a, oreal b) { g_oracle_ops[OC_MINMAX]++; return (b.v < a.v) ? b : a; }
inline oreal osin(oreal a) { return oreal(std::sin(a.v)); }
inline oreal ocos(oreal a) { return oreal(std::cos(a.v)); }
#endif
