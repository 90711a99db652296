#ifndef SHIM_BOOLEAN_H
#define SHIM_BOOLEAN_H
#endif
