// Regression.hpp — least squares through the origin, y = k x (long double, as the reference).
#ifndef REGRESSION_HPP
#define REGRESSION_HPP

class UnbiasedLinearRegression {
 private:
  bool is_solved;
  long double k;

 public:
  UnbiasedLinearRegression();
  void solve(long double* x, long double* y, unsigned int len);
  long double get_k();
};

#endif
