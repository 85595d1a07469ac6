/* Test double of the MATLAB C matrix API: the handful of types and calls the
 * MEX gateway uses, so that it compiles and runs without MATLAB (test
 * infrastructure only; tests/test_mex_gateway.py). */
#ifndef FMF_MOCK_MATRIX_H
#define FMF_MOCK_MATRIX_H
#include <stddef.h>

typedef size_t mwSize;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7, mxINT32_CLASS = 12 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;

size_t mxGetNumberOfElements(const mxArray *a);
double mxGetScalar(const mxArray *a);
mxClassID mxGetClassID(const mxArray *a);
int mxIsComplex(const mxArray *a);
void *mxGetData(const mxArray *a);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity cplx);
#endif
