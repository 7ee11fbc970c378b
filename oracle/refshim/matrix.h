/* Minimal declarations of the MATLAB C matrix API (public interface,
 * interleaved-complex form) for compiling QSpace's MEX sources against the
 * project's fake runtime (fakemx.cpp).  Test infrastructure only. */
#ifndef FAKEMX_MATRIX_H
#define FAKEMX_MATRIX_H
#include <float.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef size_t mwSize;
typedef size_t mwIndex;
typedef ptrdiff_t mwSignedIndex;
typedef struct mxArray_tag mxArray;
#ifdef __cplusplus
typedef char16_t mxChar;
#else
typedef uint16_t mxChar;
#endif
typedef bool mxLogical;
typedef double mxDouble;
typedef float mxSingle;
typedef int8_t mxInt8;
typedef uint8_t mxUint8;
typedef int16_t mxInt16;
typedef uint16_t mxUint16;
typedef int32_t mxInt32;
typedef uint32_t mxUint32;
typedef int64_t mxInt64;
typedef uint64_t mxUint64;
typedef struct { mxDouble real, imag; } mxComplexDouble;
/* fixed-width names of MATLAB's tmwtypes.h */
typedef int8_t int8_T;
typedef uint8_t uint8_T;
typedef int16_t int16_T;
typedef uint16_t uint16_T;
typedef int32_t int32_T;
typedef uint32_t uint32_T;
typedef int64_t int64_T;
typedef uint64_t uint64_T;
typedef double real_T;
typedef bool boolean_T;

typedef enum {
  mxUNKNOWN_CLASS = 0, mxCELL_CLASS, mxSTRUCT_CLASS, mxLOGICAL_CLASS, mxCHAR_CLASS, mxVOID_CLASS,
  mxDOUBLE_CLASS, mxSINGLE_CLASS, mxINT8_CLASS, mxUINT8_CLASS, mxINT16_CLASS, mxUINT16_CLASS,
  mxINT32_CLASS, mxUINT32_CLASS, mxINT64_CLASS, mxUINT64_CLASS, mxFUNCTION_CLASS, mxOPAQUE_CLASS,
  mxOBJECT_CLASS
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

#ifdef __cplusplus
extern "C" {
#endif
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID cls, mxComplexity c);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c);
mxArray *mxCreateCellMatrix(mwSize m, mwSize n);
mxArray *mxCreateCellArray(mwSize ndim, const mwSize *dims);
mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **fieldnames);
mxArray *mxCreateStructArray(mwSize ndim, const mwSize *dims, int nfields, const char **fieldnames);
mxArray *mxCreateString(const char *str);
mxArray *mxCreateCharArray(mwSize ndim, const mwSize *dims);
mxArray *mxCreateSparse(mwSize m, mwSize n, mwSize nzmax, mxComplexity c);
mxArray *mxCreateLogicalMatrix(mwSize m, mwSize n);
mxArray *mxCreateLogicalScalar(bool v);
mxArray *mxDuplicateArray(const mxArray *a);
void mxDestroyArray(mxArray *a);
int mxAddField(mxArray *a, const char *name);
void mxRemoveField(mxArray *a, int k);
mxArray *mxGetCell(const mxArray *a, mwIndex i);
void mxSetCell(mxArray *a, mwIndex i, mxArray *v);
mxChar *mxGetChars(const mxArray *a);
mxClassID mxGetClassID(const mxArray *a);
const char *mxGetClassName(const mxArray *a);
mxComplexDouble *mxGetComplexDoubles(const mxArray *a);
void *mxGetData(const mxArray *a);
void mxSetData(mxArray *a, void *d);
const mwSize *mxGetDimensions(const mxArray *a);
mxDouble *mxGetDoubles(const mxArray *a);
double *mxGetPr(const mxArray *a);
double mxGetScalar(const mxArray *a);
mxArray *mxGetField(const mxArray *a, mwIndex i, const char *name);
void mxSetField(mxArray *a, mwIndex i, const char *name, mxArray *v);
mxArray *mxGetFieldByNumber(const mxArray *a, mwIndex i, int k);
void mxSetFieldByNumber(mxArray *a, mwIndex i, int k, mxArray *v);
const char *mxGetFieldNameByNumber(const mxArray *a, int k);
int mxGetFieldNumber(const mxArray *a, const char *name);
mxInt8 *mxGetInt8s(const mxArray *a);
mxUint8 *mxGetUint8s(const mxArray *a);
mxInt16 *mxGetInt16s(const mxArray *a);
mxUint16 *mxGetUint16s(const mxArray *a);
mxInt32 *mxGetInt32s(const mxArray *a);
mxUint32 *mxGetUint32s(const mxArray *a);
mxInt64 *mxGetInt64s(const mxArray *a);
mxUint64 *mxGetUint64s(const mxArray *a);
mwIndex *mxGetIr(const mxArray *a);
mwIndex *mxGetJc(const mxArray *a);
mxLogical *mxGetLogicals(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
void mxSetM(mxArray *a, mwSize m);
void mxSetN(mxArray *a, mwSize n);
mwSize mxGetNumberOfDimensions(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
int mxGetNumberOfFields(const mxArray *a);
mwSize mxGetNzmax(const mxArray *a);
size_t mxGetElementSize(const mxArray *a);
int mxGetString(const mxArray *a, char *buf, mwSize buflen);
char *mxArrayToString(const mxArray *a);
bool mxIsCell(const mxArray *a);
bool mxIsChar(const mxArray *a);
bool mxIsComplex(const mxArray *a);
bool mxIsDouble(const mxArray *a);
bool mxIsSingle(const mxArray *a);
bool mxIsEmpty(const mxArray *a);
bool mxIsInt8(const mxArray *a);
bool mxIsLogical(const mxArray *a);
bool mxIsNumeric(const mxArray *a);
bool mxIsSparse(const mxArray *a);
bool mxIsStruct(const mxArray *a);
bool mxIsClass(const mxArray *a, const char *name);
int mxSetClassName(mxArray *a, const char *name);
int mxSetDimensions(mxArray *a, const mwSize *dims, mwSize ndim);
void *mxMalloc(size_t n);
void *mxCalloc(size_t n, size_t s);
void *mxRealloc(void *p, size_t n);
void mxFree(void *p);
#ifdef __cplusplus
}
#endif
#endif
