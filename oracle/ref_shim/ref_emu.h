#ifndef SHIM_REF_EMU_H
#define SHIM_REF_EMU_H
enum
{
    REF_CU_NONE = 0,
    REF_CU_PR_PULL_F32, REF_CU_PR_PUSH_F32,
    REF_CU_PR_PULL_U64, REF_CU_PR_PULL_U32, REF_CU_PR_PULL_U16, REF_CU_PR_PULL_U8,
    REF_CU_BFS_BOTTOM_UP, REF_CU_SPMV_PULL_F32
};
extern int ref_emu_cu_kind;
struct GraphCSR;
void ref_emu_set_graph(struct GraphCSR *graph);
#endif
