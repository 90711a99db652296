#ifndef SHIM_LIBCXL_H
#define SHIM_LIBCXL_H
struct cxl_afu_h { int unused; };
#endif
