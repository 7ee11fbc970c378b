#include "blas.h"
