/*
 * fmf_gb300_mex.c -- MATLAB MEX gateway of the GPU matched filter.
 *
 * Takes the place of the reference's MEX gateways (src/matched_filter_mex.c,
 * src/matched_filter_precise_mex.c), which call the CPU library: this one
 * calls libfmf_gb300 (include/fmf_gb300.h), so a MATLAB user runs the same
 * search on the GPU.  MATLAB stores arrays column-major, so the reference's
 * MATLAB layouts -- templates [time x components x stations x templates],
 * data [time x components x stations], moveouts and weights [components x
 * stations x templates] -- are in memory exactly the library's row-major
 * (T, S, C, L), (S, C, N) and (T, S, C): the gateway passes the pointers
 * through.
 *
 *   cc_sum = fmf_gb300_mex(templates, sum_square_templates, moveouts, data,
 *                          weights, step, n_samples_template, n_samples_data,
 *                          n_templates, n_stations, n_components, n_corr
 *                          [, normalize [, precision]])
 *
 * The twelve required arguments are the reference gateway's, in its order
 * (single, single, int32, single, single, then scalars); normalize is 0
 * ('short', default) or 1 ('full'), precision an FMF_PREC_* code (default
 * FMF_PREC_FP32).  The output is a single column of n_corr * n_templates
 * network sums, template-major (reshape(cc_sum, [], n_templates) in MATLAB
 * gives [lags x templates], as the reference wrapper does).
 *
 * Unlike the reference gateways, every array's class and element count is
 * checked before the call (a wrong class would be read as the wrong type),
 * and a failure of the library is reported through mexErrMsgIdAndTxt with
 * the library's message.
 *
 * Build (MATLAB's mex, against the in-tree library):
 *   mex -I<repo>/include -L<repo>/fast_matched_filter_gb300/lib -lfmf_gb300 fmf_gb300_mex.c
 */
#include <stddef.h>
#include <stdio.h>

#include <mex.h>
#include <matrix.h>

#include "fmf_gb300.h"

#define FMF_MEX_ID "fmf_gb300:mex"

/* Scalar argument i as a non-negative size; raises on anything else. */
static size_t size_arg(const mxArray *a, int i)
{
    if (mxGetNumberOfElements(a) != 1)
        mexErrMsgIdAndTxt(FMF_MEX_ID, "argument %d must be a scalar", i + 1);
    const double v = mxGetScalar(a);
    if (!(v >= 0.0) || v != (double)(size_t)v)
        mexErrMsgIdAndTxt(FMF_MEX_ID, "argument %d must be a non-negative integer", i + 1);
    return (size_t)v;
}

/* Array argument i of the given class and element count. */
static void *array_arg(const mxArray *a, int i, mxClassID cls, const char *cls_name, size_t count)
{
    if (mxGetClassID(a) != cls || mxIsComplex(a))
        mexErrMsgIdAndTxt(FMF_MEX_ID, "argument %d must be a real %s array", i + 1, cls_name);
    if ((size_t)mxGetNumberOfElements(a) != count)
        mexErrMsgIdAndTxt(FMF_MEX_ID, "argument %d has %zu elements, %zu expected", i + 1,
                          (size_t)mxGetNumberOfElements(a), count);
    return mxGetData(a);
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs < 12 || nrhs > 14)
        mexErrMsgIdAndTxt(FMF_MEX_ID,
                          "12 to 14 inputs: templates, sum_square_templates, moveouts, data, weights, "
                          "step, n_samples_template, n_samples_data, n_templates, n_stations, "
                          "n_components, n_corr [, normalize [, precision]]");
    if (nlhs > 1)
        mexErrMsgIdAndTxt(FMF_MEX_ID, "one output: cc_sum");
    const size_t step = size_arg(prhs[5], 5), L = size_arg(prhs[6], 6), N = size_arg(prhs[7], 7);
    const size_t T = size_arg(prhs[8], 8), S = size_arg(prhs[9], 9), C = size_arg(prhs[10], 10);
    const size_t n_corr = size_arg(prhs[11], 11);
    const int normalize = nrhs > 12 ? (int)size_arg(prhs[12], 12) : 0;
    const int precision = nrhs > 13 ? (int)size_arg(prhs[13], 13) : FMF_PREC_FP32;
    const size_t tsc = T * S * C;
    const float *tpl = (const float *)array_arg(prhs[0], 0, mxSINGLE_CLASS, "single", tsc * L);
    const float *sst = (const float *)array_arg(prhs[1], 1, mxSINGLE_CLASS, "single", tsc);
    const int *mo = (const int *)array_arg(prhs[2], 2, mxINT32_CLASS, "int32", tsc);
    const float *data = (const float *)array_arg(prhs[3], 3, mxSINGLE_CLASS, "single", S * C * N);
    const float *w = (const float *)array_arg(prhs[4], 4, mxSINGLE_CLASS, "single", tsc);

    const mwSize n_out = (mwSize)(n_corr * T);
    plhs[0] = mxCreateNumericArray(1, &n_out, mxSINGLE_CLASS, mxREAL);
    float *cc = (float *)mxGetData(plhs[0]);
    const int st = fmf_matched_filter_ex(tpl, sst, mo, data, w, step, L, N, T, S, C, n_corr, cc,
                                         normalize, 1, precision, 0, NULL);
    if (st != FMF_OK) {
        char msg[512];
        fmf_last_error(msg, sizeof msg);
        mexErrMsgIdAndTxt(FMF_MEX_ID, "fmf_matched_filter_ex failed (status %d): %s", st, msg);
    }
}
