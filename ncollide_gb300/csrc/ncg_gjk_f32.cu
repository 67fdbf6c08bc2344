// ncg_gjk_f32.cu — the GJK stage in the reference's f32 arithmetic (namespace
// f32a): ncg_gjk.cu compiled with NCG_REAL_F32.
#define NCG_REAL_F32 1
#include "ncg_gjk.cu"
