// fk_inst_ds.cu -- kernel instances for one precision (see fk_inst.cuh).
#define FK_PREC_NAME ds
#define FK_SYS_R fk::SysDSR
#define FK_SYS_C fk::SysDSC
#include "fk_inst.cuh"
