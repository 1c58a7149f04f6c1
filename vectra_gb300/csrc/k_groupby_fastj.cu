// k_groupby_fastj.cu -- the join instantiations of the specialised
// aggregation kernel (a second translation unit so the build compiles them
// in parallel with the others).  Join semantics: join_probe_one
// (src/join.c:262-480); NA keys never match (src/join.c:77-113).
#define VG_FAST_PART 1
#include "k_groupby_fast.cu"
