/* Declarations of the MATLAB MEX API functions the gateways use (names and
 * signatures as MATLAB's mex.h declares them), so that the gateways can be
 * compiled for a syntax and type check where MATLAB is not installed.  Not a
 * MEX implementation: nothing is linked against it. */
#pragma once
#include <stddef.h>
#include <stdio.h>
typedef size_t mwSize;
typedef size_t mwIndex;
typedef struct mxArray_tag mxArray;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
typedef enum { mxUINT64_CLASS } mxClassID;
extern "C" {
void mexErrMsgIdAndTxt(const char*, const char*, ...);
bool mxIsUint64(const mxArray*);
bool mxIsDouble(const mxArray*);
bool mxIsComplex(const mxArray*);
bool mxIsSparse(const mxArray*);
void* mxGetData(const mxArray*);
double* mxGetPr(const mxArray*);
mwSize mxGetM(const mxArray*);
mwSize mxGetN(const mxArray*);
mwIndex* mxGetJc(const mxArray*);
mwIndex* mxGetIr(const mxArray*);
size_t mxGetNumberOfElements(const mxArray*);
double mxGetScalar(const mxArray*);
mxArray* mxCreateDoubleMatrix(mwSize, mwSize, mxComplexity);
mxArray* mxCreateNumericMatrix(mwSize, mwSize, mxClassID, mxComplexity);
bool mxIsStruct(const mxArray*);
bool mxIsChar(const mxArray*);
mxArray* mxGetField(const mxArray*, mwIndex, const char*);
char* mxArrayToString(const mxArray*);
void mxFree(void*);
}
