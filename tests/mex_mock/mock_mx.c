/* Test double of the MATLAB runtime for the MEX gateway: arrays that wrap
 * caller memory, an error call that returns to the harness by longjmp, and
 * mock_call(), which runs mexFunction and hands its output or its error
 * message back (test infrastructure only). */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

struct mxArray_tag {
    mxClassID cls;
    size_t n;
    void *data;
    int owned;
};

static jmp_buf g_jmp;
static char g_msg[1024];

size_t mxGetNumberOfElements(const mxArray *a) { return a->n; }
mxClassID mxGetClassID(const mxArray *a) { return a->cls; }
int mxIsComplex(const mxArray *a) { (void)a; return 0; }
void *mxGetData(const mxArray *a) { return a->data; }

double mxGetScalar(const mxArray *a)
{
    switch (a->cls) {
    case mxDOUBLE_CLASS: return ((const double *)a->data)[0];
    case mxSINGLE_CLASS: return ((const float *)a->data)[0];
    case mxINT32_CLASS: return ((const int *)a->data)[0];
    default: return 0.0;
    }
}

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity cplx)
{
    (void)cplx;
    size_t n = 1;
    for (mwSize i = 0; i < ndim; i++)
        n *= dims[i];
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->cls = cls;
    a->n = n;
    a->data = calloc(n ? n : 1, cls == mxDOUBLE_CLASS ? 8 : 4);
    a->owned = 1;
    return a;
}

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...)
{
    va_list ap;
    int k = snprintf(g_msg, sizeof g_msg, "%s: ", id);
    va_start(ap, fmt);
    vsnprintf(g_msg + k, sizeof g_msg - (size_t)k, fmt, ap);
    va_end(ap);
    longjmp(g_jmp, 1);
}

/* harness API */
mxArray *mock_array(int cls, size_t n, void *data)
{
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->cls = (mxClassID)cls;
    a->n = n;
    a->data = data;
    return a;
}

void mock_free(mxArray *a)
{
    if (a && a->owned)
        free(a->data);
    free(a);
}

/* 0: success, the output's elements copied to out (at most out_cap floats,
 * *out_n set); 1: mexErrMsgIdAndTxt was called, its message in msg. */
int mock_call(int nlhs, int nrhs, const mxArray **prhs, float *out, size_t out_cap, size_t *out_n,
              char *msg, size_t msg_len)
{
    static mxArray *plhs[1];  /* not a local: its value must survive the longjmp */
    plhs[0] = NULL;
    if (setjmp(g_jmp)) {
        snprintf(msg, msg_len, "%s", g_msg);
        mock_free(plhs[0]);
        return 1;
    }
    mexFunction(nlhs, plhs, nrhs, prhs);
    *out_n = plhs[0] ? plhs[0]->n : 0;
    if (plhs[0] && out)
        memcpy(out, plhs[0]->data, (plhs[0]->n < out_cap ? plhs[0]->n : out_cap) * sizeof(float));
    mock_free(plhs[0]);
    return 0;
}
