#ifndef SHIM_REORDER_H
#define SHIM_REORDER_H
#endif
