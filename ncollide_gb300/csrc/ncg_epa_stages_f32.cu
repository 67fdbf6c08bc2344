// ncg_epa_stages_f32.cu — the EPA stages in the reference's f32 arithmetic
// (namespace f32a): ncg_epa_stages.cu compiled with NCG_REAL_F32.
#define NCG_REAL_F32 1
#include "ncg_epa_stages.cu"
