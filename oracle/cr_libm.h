/* Test infrastructure only.  Force-included (gcc -include) when epic_port.c is compiled as
 * libepicport_cr.so: it routes the restatement's log, exp and pow to the correctly rounded
 * functions of cr_libm.cpp, so that the CPU restatement and the CUDA kernels share their
 * libm rounding and can be compared bit for bit (atan and cos only in the turbulence closure).  libepicport.so, the parity oracle proper,
 * keeps the host's glibc, as the reference does. */
#include <math.h>
double epic_cr_log(double x);
double epic_cr_exp(double x);
double epic_cr_pow(double x, double y);
double epic_cr_atan(double x);
double epic_cr_cos(double x);
/* the turbulence closure's atan and cos (epic_port.c names them through these macros, so the
 * grid tables, computed with the host's trigonometry on both sides, keep glibc's) */
#define EP_TURB_ATAN epic_cr_atan
#define EP_TURB_COS epic_cr_cos
#define log epic_cr_log
#define exp epic_cr_exp
#define pow epic_cr_pow
