/*
 * Minimal stand-in for MATLAB's MEX C API, written for this project's oracle.
 *
 * TEST INFRASTRUCTURE ONLY: it lets the reference's C++ MEX kernels
 * (src/MEXfuncs/*.cpp) and this project's own MEX gateway be compiled with
 * g++ and driven from Python (ctypes) without MATLAB.  Only the documented
 * MATLAB C API names that those sources use are provided.  Arrays are always
 * column-major, as in MATLAB.  mexErrMsgIdAndTxt throws a C++ exception that
 * the shim's call wrapper (shim_call) turns into an error string.
 */
#ifndef SGLD_MEXSHIM_MEX_H
#define SGLD_MEXSHIM_MEX_H
#include "matrix.h"

#ifdef __cplusplus
extern "C" {
#endif
/* Every MEX translation unit defines this entry point.  The oracle build
 * renames it per file with -DmexFunction=<name>. */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
void mexWarnMsgIdAndTxt(const char *id, const char *fmt, ...);
int mexPrintf(const char *fmt, ...);
/* Registers the function MATLAB calls when the MEX file is cleared; the shim
 * runs it from shim_run_at_exit(). */
int mexAtExit(void (*exit_fcn)(void));
#ifdef __cplusplus
}
#endif
#endif
