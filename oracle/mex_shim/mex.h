/*
 * Minimal stand-in for MATLAB's mex.h (test infrastructure only).
 *
 * It provides just the types and calls that the reference's MEX ray tracers
 * (Matlab/RayTracing3DTOF.cpp, Matlab/RayTracing3D.cpp) use, so those files
 * compile unmodified with g++ into oracle/_ref/ and can be driven from Python
 * through mex_entry.c.  Matrices are column vectors/row vectors of double,
 * single or int32; errors jump back to the entry point.
 */
#ifndef SSS_MEX_SHIM_H
#define SSS_MEX_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7, mxINT32_CLASS = 12 } mxClassID;
typedef enum { mxREAL = 0 } mxComplexity;

typedef struct mxArray_tag {
    size_t m, n;
    mxClassID cls;
    void *data;
} mxArray;

size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
int mxIsClass(const mxArray *a, const char *name);
double *mxGetPr(const mxArray *a);
void *mxGetData(const mxArray *a);
mxArray *mxCreateNumericMatrix(size_t m, size_t n, mxClassID cls, mxComplexity cplx);
void *mxRealloc(void *p, size_t bytes);
void mxSetM(mxArray *a, size_t m);
void mxSetN(mxArray *a, size_t n);
void mxSetData(mxArray *a, void *p);
void mexErrMsgTxt(const char *msg);

/* the gateway every MEX file defines; declared here so it gets C linkage */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

#ifdef __cplusplus
}
#endif

#endif
