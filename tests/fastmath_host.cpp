// Host build of the kernels' table-driven exp/exp10/log/rcp/atan/rsqrt (same source as the
// device build), exported for tests/test_fastmath.py.
#include "../dwarf-p-ice3_gb300/csrc/fastmath.cuh"

extern "C" void fm_eval(int fn, const double *x, double *y, long n)
{
  for (long i = 0; i < n; ++i)
    y[i] = fn == 0 ? fm::fexp(x[i]) : fn == 1 ? fm::fexp10(x[i]) : fn == 2 ? fm::flog(x[i])
         : fn == 3 ? fm::frcp(x[i]) : fn == 4 ? fm::fatan(x[i]) : fm::frsqrt(x[i]);
}

// a / b by fdiv_rn (mode 0) or fdiv_rn2 with the numerators a and 2.5 a (mode 1, both returned)
extern "C" void fm_div(int mode, const double *a, const double *b, double *q, double *q2, long n)
{
  for (long i = 0; i < n; ++i) {
    if (mode == 0) q[i] = fm::fdiv_rn(a[i], b[i]);
    else fm::fdiv_rn2(a[i], 2.5 * a[i], b[i], q[i], q2[i]);
  }
}
