// fk_inst_f64.cu -- kernel instances for one precision (see fk_inst.cuh).
#define FK_PREC_NAME f64
#define FK_SYS_R fk::SysF64R
#define FK_SYS_C fk::SysF64C
#include "fk_inst.cuh"
