// Host build of the kernels' table-driven exp/exp10/log/rcp/atan/rsqrt (same source as the
// device build), exported for tests/test_fastmath.py.
#include "../dwarf-p-ice3_gb300/csrc/fastmath.cuh"

extern "C" void fm_eval(int fn, const double *x, double *y, long n)
{
  for (long i = 0; i < n; ++i)
    y[i] = fn == 0 ? fm::fexp(x[i]) : fn == 1 ? fm::fexp10(x[i]) : fn == 2 ? fm::flog(x[i])
         : fn == 3 ? fm::frcp(x[i]) : fn == 4 ? fm::fatan(x[i]) : fm::frsqrt(x[i]);
}
