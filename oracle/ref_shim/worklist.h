#ifndef SHIM_WORKLIST_H
#define SHIM_WORKLIST_H
#endif
