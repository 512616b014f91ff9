/* Minimal mxArray model for the oracle's MEX shim (see mex.h). */
#ifndef SGLD_MEXSHIM_MATRIX_H
#define SGLD_MEXSHIM_MATRIX_H
#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

typedef size_t mwSize;
typedef size_t mwIndex;
typedef ptrdiff_t mwSignedIndex;
typedef int32_t int32_T;
typedef uint32_t uint32_T;
typedef int64_t int64_T;
typedef double real_T;

typedef enum {
    mxUNKNOWN_CLASS = 0, mxCELL_CLASS, mxSTRUCT_CLASS, mxLOGICAL_CLASS,
    mxCHAR_CLASS, mxVOID_CLASS, mxDOUBLE_CLASS, mxSINGLE_CLASS, mxINT8_CLASS,
    mxUINT8_CLASS, mxINT16_CLASS, mxUINT16_CLASS, mxINT32_CLASS,
    mxUINT32_CLASS, mxINT64_CLASS, mxUINT64_CLASS
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct mxArray_tag mxArray;

#ifdef __cplusplus
extern "C" {
#endif
double *mxGetPr(const mxArray *a);
void *mxGetData(const mxArray *a);
mwSize mxGetM(const mxArray *a);
mwSize mxGetN(const mxArray *a);
mwSize mxGetNumberOfElements(const mxArray *a);
mwSize mxGetNumberOfDimensions(const mxArray *a);
const mwSize *mxGetDimensions(const mxArray *a);
mxArray *mxGetCell(const mxArray *a, mwIndex i);
double mxGetScalar(const mxArray *a);
mwIndex *mxGetIr(const mxArray *a);
mwIndex *mxGetJc(const mxArray *a);
bool mxIsDouble(const mxArray *a);
bool mxIsSingle(const mxArray *a);
bool mxIsInt32(const mxArray *a);
bool mxIsLogical(const mxArray *a);
bool mxIsChar(const mxArray *a);
bool mxIsComplex(const mxArray *a);
bool mxIsCell(const mxArray *a);
bool mxIsSparse(const mxArray *a);
mxClassID mxGetClassID(const mxArray *a);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity c);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c);
mxArray *mxCreateLogicalMatrix(mwSize m, mwSize n);
mxArray *mxCreateString(const char *s);
int mxGetString(const mxArray *a, char *buf, mwSize buflen);
void *mxMalloc(size_t n);
void *mxCalloc(size_t n, size_t size);
void mxFree(void *p);
void mxDestroyArray(mxArray *a);
#ifdef __cplusplus
}
#endif
#endif
