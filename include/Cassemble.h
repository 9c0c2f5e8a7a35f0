/* Cassemble.h - the reference's header name for this library's C++ Cassemble entry points.
 * Code written against the reference (its cython/nlfem.pyx through include/Cassemble.pxd,
 * `cdef extern from "Cassemble.h"`) finds the declarations of Cassemble_compat.h here and links
 * against libnlfem_gpu.so, with no change to that code. */
#ifndef NLFEM_CASSEMBLE_H
#define NLFEM_CASSEMBLE_H
#include "Cassemble_compat.h"
#endif
