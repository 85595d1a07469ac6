/* Test double of MATLAB's mex.h (see matrix.h). */
#ifndef FMF_MOCK_MEX_H
#define FMF_MOCK_MEX_H
#include "matrix.h"

void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
#endif
