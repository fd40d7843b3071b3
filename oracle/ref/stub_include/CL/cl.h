/* Stand-in for the OpenCL types Yune's host headers use (include/CL_headers.h).
 * TEST INFRASTRUCTURE: lets the reference BVH builder compile without an OpenCL SDK. */
#ifndef YREF_STUB_CL_H
#define YREF_STUB_CL_H
typedef int cl_int;
typedef unsigned int cl_uint;
typedef float cl_float;
typedef union alignas(16) { cl_float s[4]; struct { cl_float x, y, z, w; }; } cl_float4;
#endif
