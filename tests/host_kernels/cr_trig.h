// cr_trig.h -- force-included into the host class for the stroke check: its
// round joins then take acos and tan in double rounded to float, as the
// device does (the oracle's trig="cr" variant does the same).
#include <cmath>
#include <math.h>
static inline float cr_acosf(float x) { return static_cast<float>(std::acos(static_cast<double>(x))); }
static inline float cr_tanf(float x) { return static_cast<float>(std::tan(static_cast<double>(x))); }
#define acosf cr_acosf
#define tanf cr_tanf
