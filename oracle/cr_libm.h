/* Test infrastructure only.  Force-included (gcc -include) when epic_port.c is compiled as
 * libepicport_cr.so: it routes the restatement's log, exp and pow to the correctly rounded
 * functions of cr_libm.cpp, so that the CPU restatement and the CUDA kernels share their
 * libm rounding and can be compared bit for bit.  libepicport.so, the parity oracle proper,
 * keeps the host's glibc, as the reference does. */
#include <math.h>
double epic_cr_log(double x);
double epic_cr_exp(double x);
double epic_cr_pow(double x, double y);
#define log epic_cr_log
#define exp epic_cr_exp
#define pow epic_cr_pow
