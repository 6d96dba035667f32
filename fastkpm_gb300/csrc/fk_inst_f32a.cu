// fk_inst_f32a.cu -- kernel instances of the FP32 systems with FP64 accumulators (see fk_inst.cuh).
#define FK_PREC_NAME f32a
#define FK_SYS_R fk::SysF32RA
#define FK_SYS_C fk::SysF32CA
#include "fk_inst.cuh"
