/*
 * Implementation of the oracle's minimal MEX API stand-in (see mex.h).
 *
 * TEST INFRASTRUCTURE ONLY.  Besides the MATLAB-named functions, it exports a
 * few shim_* helpers so that Python (ctypes) can build mxArrays, call a
 * mexFunction-style entry point and read the results back:
 *   shim_new_numeric(cls, m, n, data)  column-major copy of data
 *   shim_new_nd(cls, ndim, dims, data)
 *   shim_new_cell(n), shim_cell_set(cell, i, elem)   (cell takes ownership)
 *   shim_new_sparse(m, n, nnz, jc, ir, pr)           CSC, 0-based ir
 *   shim_new_string(s)
 *   shim_call(fn, nlhs, plhs, nrhs, prhs, err, errlen) -> 0 or 1 on error
 *   shim_destroy(a)
 */
#include "mex.h"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

struct mxArray_tag {
    mxClassID cls = mxUNKNOWN_CLASS;
    std::vector<mwSize> dims;
    void *data = nullptr;          // dense payload (or sparse pr)
    size_t elsize = 0;
    bool sparse = false;
    std::vector<mwIndex> ir, jc;   // sparse structure (CSC)
    std::vector<mxArray *> cells;  // cell payload (owned)
};

namespace {
struct MexError : std::runtime_error {
    explicit MexError(const std::string &s) : std::runtime_error(s) {}
};

size_t class_size(mxClassID c) {
    switch (c) {
        case mxDOUBLE_CLASS: case mxINT64_CLASS: case mxUINT64_CLASS: return 8;
        case mxSINGLE_CLASS: case mxINT32_CLASS: case mxUINT32_CLASS: return 4;
        case mxINT16_CLASS: case mxUINT16_CLASS: case mxCHAR_CLASS: return 2;
        case mxINT8_CLASS: case mxUINT8_CLASS: case mxLOGICAL_CLASS: return 1;
        default: return 0;
    }
}

mwSize numel(const mxArray *a) {
    mwSize n = 1;
    for (mwSize d : a->dims) n *= d;
    return n;
}

mxArray *alloc_dense(mxClassID cls, const std::vector<mwSize> &dims) {
    auto *a = new mxArray_tag;
    a->cls = cls;
    a->dims = dims;
    while (a->dims.size() < 2) a->dims.push_back(1);
    a->elsize = class_size(cls);
    size_t bytes = numel(a) * a->elsize;
    a->data = std::calloc(bytes ? bytes : 1, 1);
    return a;
}
}  // namespace

extern "C" {

double *mxGetPr(const mxArray *a) { return static_cast<double *>(a->data); }
void *mxGetData(const mxArray *a) { return a->data; }
mwSize mxGetM(const mxArray *a) { return a->dims[0]; }
mwSize mxGetN(const mxArray *a) {
    mwSize n = 1;
    for (size_t i = 1; i < a->dims.size(); ++i) n *= a->dims[i];
    return n;
}
mwSize mxGetNumberOfElements(const mxArray *a) { return numel(a); }
mwSize mxGetNumberOfDimensions(const mxArray *a) { return a->dims.size(); }
const mwSize *mxGetDimensions(const mxArray *a) { return a->dims.data(); }
mxArray *mxGetCell(const mxArray *a, mwIndex i) {
    if (a->cls != mxCELL_CLASS || i >= a->cells.size()) return nullptr;
    return a->cells[i];
}
double mxGetScalar(const mxArray *a) {
    switch (a->cls) {
        case mxDOUBLE_CLASS: return static_cast<double *>(a->data)[0];
        case mxSINGLE_CLASS: return static_cast<float *>(a->data)[0];
        case mxINT32_CLASS: return static_cast<int32_t *>(a->data)[0];
        case mxUINT32_CLASS: return static_cast<uint32_t *>(a->data)[0];
        case mxINT64_CLASS: return (double)static_cast<int64_t *>(a->data)[0];
        case mxUINT8_CLASS: case mxLOGICAL_CLASS: return static_cast<uint8_t *>(a->data)[0];
        default: return 0.0;
    }
}
mwIndex *mxGetIr(const mxArray *a) { return const_cast<mwIndex *>(a->ir.data()); }
mwIndex *mxGetJc(const mxArray *a) { return const_cast<mwIndex *>(a->jc.data()); }
bool mxIsDouble(const mxArray *a) { return a->cls == mxDOUBLE_CLASS; }
bool mxIsSingle(const mxArray *a) { return a->cls == mxSINGLE_CLASS; }
bool mxIsInt32(const mxArray *a) { return a->cls == mxINT32_CLASS; }
bool mxIsLogical(const mxArray *a) { return a->cls == mxLOGICAL_CLASS; }
bool mxIsChar(const mxArray *a) { return a->cls == mxCHAR_CLASS; }
bool mxIsComplex(const mxArray *) { return false; }
bool mxIsCell(const mxArray *a) { return a->cls == mxCELL_CLASS; }
bool mxIsSparse(const mxArray *a) { return a->sparse; }
mxClassID mxGetClassID(const mxArray *a) { return a->cls; }

mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity) {
    return alloc_dense(mxDOUBLE_CLASS, {m, n});
}
mxArray *mxCreateDoubleScalar(double v) {
    mxArray *a = alloc_dense(mxDOUBLE_CLASS, {1, 1});
    static_cast<double *>(a->data)[0] = v;
    return a;
}
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity) {
    return alloc_dense(cls, std::vector<mwSize>(dims, dims + ndim));
}
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity) {
    return alloc_dense(cls, {m, n});
}
mxArray *mxCreateLogicalMatrix(mwSize m, mwSize n) { return alloc_dense(mxLOGICAL_CLASS, {m, n}); }
mxArray *mxCreateString(const char *s) {
    size_t n = std::strlen(s);
    mxArray *a = alloc_dense(mxCHAR_CLASS, {1, n});
    auto *p = static_cast<uint16_t *>(a->data);
    for (size_t i = 0; i < n; ++i) p[i] = (unsigned char)s[i];
    return a;
}
int mxGetString(const mxArray *a, char *buf, mwSize buflen) {
    if (a->cls != mxCHAR_CLASS || buflen == 0) return 1;
    mwSize n = numel(a);
    auto *p = static_cast<uint16_t *>(a->data);
    mwSize k = 0;
    for (; k < n && k + 1 < buflen; ++k) buf[k] = (char)p[k];
    buf[k] = 0;
    return k < n ? 1 : 0;
}
void *mxMalloc(size_t n) { return std::malloc(n ? n : 1); }
void *mxCalloc(size_t n, size_t size) { return std::calloc(n ? n : 1, size ? size : 1); }
void mxFree(void *p) { std::free(p); }
void mxDestroyArray(mxArray *a) {
    if (!a) return;
    for (mxArray *c : a->cells) mxDestroyArray(c);
    std::free(a->data);
    delete a;
}

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...) {
    char msg[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    throw MexError(std::string(id) + ": " + msg);
}
void mexWarnMsgIdAndTxt(const char *id, const char *fmt, ...) {
    char msg[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    std::fprintf(stderr, "Warning [%s]: %s\n", id, msg);
}
int mexPrintf(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    int r = std::vprintf(fmt, ap);
    va_end(ap);
    return r;
}
static void (*g_exit_fcn)(void) = nullptr;
int mexAtExit(void (*exit_fcn)(void)) {
    g_exit_fcn = exit_fcn;
    return 0;
}

/* ---- helpers for ctypes callers ---- */
mxArray *shim_new_numeric(int cls, size_t m, size_t n, const void *src) {
    mxArray *a = alloc_dense((mxClassID)cls, {m, n});
    if (src) std::memcpy(a->data, src, m * n * a->elsize);
    return a;
}
mxArray *shim_new_nd(int cls, size_t ndim, const size_t *dims, const void *src) {
    mxArray *a = alloc_dense((mxClassID)cls, std::vector<mwSize>(dims, dims + ndim));
    if (src) std::memcpy(a->data, src, numel(a) * a->elsize);
    return a;
}
mxArray *shim_new_cell(size_t n) {
    auto *a = new mxArray_tag;
    a->cls = mxCELL_CLASS;
    a->dims = {n, 1};
    a->cells.assign(n, nullptr);
    return a;
}
void shim_cell_set(mxArray *cell, size_t i, mxArray *elem) {
    if (cell->cells[i]) mxDestroyArray(cell->cells[i]);
    cell->cells[i] = elem;
}
mxArray *shim_new_sparse(size_t m, size_t n, size_t nnz, const int64_t *jc, const int64_t *ir,
                         const double *pr) {
    auto *a = new mxArray_tag;
    a->cls = mxDOUBLE_CLASS;
    a->sparse = true;
    a->dims = {m, n};
    a->elsize = 8;
    a->jc.assign(jc, jc + n + 1);
    a->ir.assign(ir, ir + nnz);
    a->data = std::malloc((nnz ? nnz : 1) * sizeof(double));
    std::memcpy(a->data, pr, nnz * sizeof(double));
    return a;
}
mxArray *shim_new_string(const char *s) { return mxCreateString(s); }
int shim_class(const mxArray *a) { return (int)a->cls; }
size_t shim_ndim(const mxArray *a) { return a->dims.size(); }
size_t shim_dim(const mxArray *a, size_t i) { return i < a->dims.size() ? a->dims[i] : 1; }
void *shim_data(const mxArray *a) { return a->data; }
void shim_destroy(mxArray *a) { mxDestroyArray(a); }
/* what `clear mex` does to a loaded MEX file: run its mexAtExit function once */
void shim_run_at_exit(void) {
    void (*f)(void) = g_exit_fcn;
    g_exit_fcn = nullptr;
    if (f) f();
}

typedef void (*mex_entry_t)(int, mxArray **, int, const mxArray **);
int shim_call(mex_entry_t fn, int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs, char *err,
              size_t errlen) {
    try {
        fn(nlhs, plhs, nrhs, prhs);
        return 0;
    } catch (const std::exception &e) {
        if (err && errlen) {
            std::strncpy(err, e.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return 1;
    }
}
}  // extern "C"
