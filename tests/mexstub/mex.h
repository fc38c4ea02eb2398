/* Minimal declarations of the MATLAB MEX C API used by sid_gb300/matlab/sid_mex.c,
 * for a compile check of the gateway on machines without MATLAB.  Only the
 * names and argument types matter here; nothing links against these. */
#ifndef SID_TEST_MEX_STUB_H
#define SID_TEST_MEX_STUB_H
#include <stddef.h>
#include <stdbool.h>

typedef size_t mwSize;
typedef size_t mwIndex;
typedef struct mxArray_tag mxArray;
typedef bool mxLogical;
typedef enum {
    mxUNKNOWN_CLASS, mxCELL_CLASS, mxSTRUCT_CLASS, mxLOGICAL_CLASS, mxCHAR_CLASS, mxVOID_CLASS, mxDOUBLE_CLASS,
    mxSINGLE_CLASS, mxINT8_CLASS, mxUINT8_CLASS, mxINT16_CLASS, mxUINT16_CLASS, mxINT32_CLASS, mxUINT32_CLASS,
    mxINT64_CLASS, mxUINT64_CLASS
} mxClassID;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexAtExit(void (*fn)(void));
double mxGetScalar(const mxArray* a);
double* mxGetPr(const mxArray* a);
void* mxGetData(const mxArray* a);
mxLogical* mxGetLogicals(const mxArray* a);
int mxGetString(const mxArray* a, char* buf, mwSize len);
mwSize mxGetNumberOfElements(const mxArray* a);
mwSize mxGetNumberOfDimensions(const mxArray* a);
const mwSize* mxGetDimensions(const mxArray* a);
mxArray* mxGetField(const mxArray* a, mwIndex i, const char* name);
mxArray* mxGetCell(const mxArray* a, mwIndex i);
bool mxIsEmpty(const mxArray* a);
bool mxIsStruct(const mxArray* a);
bool mxIsChar(const mxArray* a);
bool mxIsSingle(const mxArray* a);
bool mxIsDouble(const mxArray* a);
bool mxIsLogical(const mxArray* a);
bool mxIsComplex(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
mxArray* mxCreateDoubleScalar(double v);
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray* mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c);
mxArray* mxCreateNumericArray(mwSize nd, const mwSize* dims, mxClassID cls, mxComplexity c);
mxArray* mxDuplicateArray(const mxArray* a);
void mxDestroyArray(mxArray* a);
void* mxMalloc(size_t n);
void mxFree(void* p);

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
#endif
