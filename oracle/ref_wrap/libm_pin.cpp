/* Pins the one platform-dependent call on the reference's path.  CFft::Init1 passes a float
 * angle to cos/sin (source/cfft.cpp:407-408), which in C++ selects the float overloads
 * cosf/sinf; their last bit differs between C libraries (glibc's cosf is not correctly rounded
 * for about 2.6% of the 16384 twiddle angles of a 32768-point transform).  Inside the reference
 * build these hidden definitions replace them with the correctly rounded value, which is what
 * the oracle restatement and the CUDA library compute on every platform.
 * TEST INFRASTRUCTURE ONLY (oracle/build_ref.sh). */
#include <math.h>
extern "C" __attribute__((visibility("hidden"))) float cosf(float x) { return (float)cos((double)x); }
extern "C" __attribute__((visibility("hidden"))) float sinf(float x) { return (float)sin((double)x); }
/* gcc merges the cos/sin pair of source/cfft.cpp:407-408 into one sincosf call. */
extern "C" __attribute__((visibility("hidden"))) void sincosf(float x, float* s, float* c) {
    *s = (float)sin((double)x);
    *c = (float)cos((double)x);
}
