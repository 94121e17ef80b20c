/* stand-in type for reconstinfo.h (TEST INFRASTRUCTURE ONLY) */
typedef int cufftHandle;
