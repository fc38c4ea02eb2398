/* Minimal declarations of MATLAB's mxGPUArray C API (Parallel Computing
 * Toolbox) used by sid_gb300/matlab/sid_mex.c, for a compile check on
 * machines without MATLAB. */
#ifndef SID_TEST_MXGPUARRAY_STUB_H
#define SID_TEST_MXGPUARRAY_STUB_H
#include "mex.h"

typedef struct mxGPUArray_tag mxGPUArray;
typedef enum { MX_GPU_INITIALIZE_VALUES, MX_GPU_DO_NOT_INITIALIZE } mxGPUInitialize;

int mxInitGPU(void);
bool mxIsGPUArray(const mxArray* a);
const mxGPUArray* mxGPUCreateFromMxArray(const mxArray* a);
mxGPUArray* mxGPUCreateGPUArray(mwSize nd, const mwSize* dims, mxClassID cls, mxComplexity c, mxGPUInitialize init);
mxGPUArray* mxGPUCopyGPUArray(const mxGPUArray* g);
mxArray* mxGPUCreateMxArrayOnGPU(const mxGPUArray* g);
mxArray* mxGPUCreateMxArrayOnCPU(const mxGPUArray* g);
void mxGPUDestroyGPUArray(const mxGPUArray* g);
mxClassID mxGPUGetClassID(const mxGPUArray* g);
void* mxGPUGetData(mxGPUArray* g);
const void* mxGPUGetDataReadOnly(const mxGPUArray* g);
const mwSize* mxGPUGetDimensions(const mxGPUArray* g);
mwSize mxGPUGetNumberOfElements(const mxGPUArray* g);
#endif
