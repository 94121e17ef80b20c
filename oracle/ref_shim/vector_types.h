/* stand-in types for reconstinfo.h (TEST INFRASTRUCTURE ONLY) */
#ifndef RVREF_VECTOR_TYPES_H_
#define RVREF_VECTOR_TYPES_H_
struct float2 { float x, y; };
typedef struct CUstream_st* cudaStream_t;
#endif
