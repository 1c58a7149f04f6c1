// k_groupby_fastj.cu -- the join instantiations of the specialised
// aggregation kernel (a second translation unit so the build compiles them
// in parallel with the others).
#define VG_FAST_PART 1
#include "k_groupby_fast.cu"
