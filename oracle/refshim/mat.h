/* Minimal MAT-file API declarations for the fake MATLAB runtime: files are
 * never read (matOpen for reading returns NULL), writes are accepted and
 * dropped.  Test infrastructure only. */
#ifndef FAKEMX_MAT_H
#define FAKEMX_MAT_H
#include "matrix.h"
typedef struct MATFile_tag MATFile;
#ifdef __cplusplus
extern "C" {
#endif
MATFile *matOpen(const char *filename, const char *mode);
int matClose(MATFile *f);
mxArray *matGetVariable(MATFile *f, const char *name);
mxArray *matGetVariableInfo(MATFile *f, const char *name);
int matPutVariable(MATFile *f, const char *name, const mxArray *a);
int matDeleteVariable(MATFile *f, const char *name);
#ifdef __cplusplus
}
#endif
#endif
