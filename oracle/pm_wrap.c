/* Test infrastructure (never linked into the product): the reference built
 * with `-Wl,--wrap=log,--wrap=sin,--wrap=cos,--wrap=sincos` (make -C oracle
 * ref_pm) calls these instead of the host libm's functions.  While
 * qs_portable_math_on is 0 they forward to libm (initMC's table construction
 * runs that way, so the tables stay the ones the deck reader builds); the
 * harness sets it to 1 before the first cycle, and from then on the
 * reference's tracking, source and collision code (MC_Segment_Outcome.cc:77-84,
 * CollisionEvent.cc:29-43, DirectionCosine.cc:5-12, MC_SourceNow.cc) use the
 * portable functions of quicksilver_gb300/csrc/portable_math.h -- the same
 * ones the oracle's and the GPU library's portable-math builds use. */
#include "../quicksilver_gb300/csrc/portable_math.h"

int qs_portable_math_on = 0;

double __real_log(double);
double __real_sin(double);
double __real_cos(double);
void __real_sincos(double, double*, double*);

double __wrap_log(double x) { return qs_portable_math_on ? qsg_log(x) : __real_log(x); }
double __wrap_sin(double x) { return qs_portable_math_on ? qsg_sin(x) : __real_sin(x); }
double __wrap_cos(double x) { return qs_portable_math_on ? qsg_cos(x) : __real_cos(x); }
void __wrap_sincos(double x, double* s, double* c)
{
    if (qs_portable_math_on) qsg_sincos(x, s, c);
    else __real_sincos(x, s, c);
}
