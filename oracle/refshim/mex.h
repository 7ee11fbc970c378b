/* Minimal MEX API declarations for the project's fake MATLAB runtime
 * (fakemx.cpp).  Test infrastructure only. */
#ifndef FAKEMX_MEX_H
#define FAKEMX_MEX_H
#include "matrix.h"
#ifdef __cplusplus
extern "C" {
#endif
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
void mexErrMsgTxt(const char *msg);
void mexWarnMsgIdAndTxt(const char *id, const char *fmt, ...);
void mexWarnMsgTxt(const char *msg);
int mexPrintf(const char *fmt, ...);
const char *mexFunctionName(void);
int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name);
int mexEvalString(const char *cmd);
const mxArray *mexGetVariablePtr(const char *ws, const char *name);
mxArray *mexGetVariable(const char *ws, const char *name);
int mexPutVariable(const char *ws, const char *name, const mxArray *a);
int mexAtExit(void (*fn)(void));
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
#ifdef __cplusplus
}
#endif
#endif
