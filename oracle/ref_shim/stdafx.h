/* Stand-in for the reference's precompiled header (TEST INFRASTRUCTURE ONLY). */
#include <afx.h>
