// fk_inst_f32.cu -- kernel instances for one precision (see fk_inst.cuh).
#define FK_PREC_NAME f32
#define FK_SYS_R fk::SysF32R
#define FK_SYS_C fk::SysF32C
#include "fk_inst.cuh"
