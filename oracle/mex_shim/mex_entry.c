/*
 * Host for the reference MEX ray tracers (test infrastructure only).
 *
 * Implements the mex.h shim and exports
 *   int ref_trace(const double grid[3], const double bounds[6],
 *                 const double line[6], double *len, int *idx,
 *                 double *samples, int cap)
 * which calls the reference's unmodified mexFunction with 1x3 / 1x6 / 1x6
 * double inputs (the MEX ABI of Matlab/RayTracing3DTOF.cpp:51-66) and copies
 * its outputs.  For RayTracing3D.cpp the first output is single precision;
 * it is widened to double here and `samples` is left untouched.
 * Returns the voxel count (0 on a miss) or -1 if the MEX code raised.
 */
#include <setjmp.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

static jmp_buf g_err;

size_t mxGetM(const mxArray *a) { return a->m; }
size_t mxGetN(const mxArray *a) { return a->n; }
int mxIsClass(const mxArray *a, const char *name)
{
    if (strcmp(name, "double") == 0) return a->cls == mxDOUBLE_CLASS;
    if (strcmp(name, "single") == 0) return a->cls == mxSINGLE_CLASS;
    if (strcmp(name, "int32") == 0) return a->cls == mxINT32_CLASS;
    return 0;
}
double *mxGetPr(const mxArray *a) { return (double *)a->data; }
void *mxGetData(const mxArray *a) { return a->data; }

static size_t elem_size(mxClassID c)
{
    return c == mxDOUBLE_CLASS ? 8 : 4;
}

mxArray *mxCreateNumericMatrix(size_t m, size_t n, mxClassID cls, mxComplexity cplx)
{
    (void)cplx;
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->m = m;
    a->n = n;
    a->cls = cls;
    a->data = calloc(m * n > 0 ? m * n : 1, elem_size(cls));
    return a;
}
void *mxRealloc(void *p, size_t bytes) { return realloc(p, bytes > 0 ? bytes : 1); }
void mxSetM(mxArray *a, size_t m) { a->m = m; }
void mxSetN(mxArray *a, size_t n) { a->n = n; }
void mxSetData(mxArray *a, void *p) { a->data = p; }
void mexErrMsgTxt(const char *msg)
{
    (void)msg;
    longjmp(g_err, 1);
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

#ifndef REF_NOUT
#define REF_NOUT 3
#endif

int ref_trace(const double grid[3], const double bounds[6], const double line[6], double *len,
              int *idx, double *samples, int cap)
{
    mxArray in0 = {1, 3, mxDOUBLE_CLASS, (void *)grid};
    mxArray in1 = {1, 6, mxDOUBLE_CLASS, (void *)bounds};
    mxArray in2 = {1, 6, mxDOUBLE_CLASS, (void *)line};
    const mxArray *prhs[3] = {&in0, &in1, &in2};
    mxArray *plhs[3] = {0, 0, 0};
    if (setjmp(g_err)) return -1;
    mexFunction(REF_NOUT, plhs, 3, prhs);
    int n = (int)(plhs[0]->m * plhs[0]->n);
    if (n > cap) n = -1;
    if (n > 0) {
        if (plhs[0]->cls == mxSINGLE_CLASS) {
            const float *f = (const float *)plhs[0]->data;
            for (int i = 0; i < n; ++i) len[i] = (double)f[i];
        } else {
            memcpy(len, plhs[0]->data, sizeof(double) * (size_t)n);
        }
        memcpy(idx, plhs[1]->data, sizeof(int) * (size_t)n);
        if (REF_NOUT == 3) memcpy(samples, plhs[2]->data, sizeof(double) * (size_t)n);
    }
    for (int i = 0; i < REF_NOUT; ++i) {
        if (plhs[i]) {
            free(plhs[i]->data);
            free(plhs[i]);
        }
    }
    return n;
}
