// The reference's generated solvers include "ops_seq.h"; this repository's minimal OPS-API
// host runtime (oracle/ops_compat.h) stands in for it.  Test infrastructure only.
#include "ops_compat.h"
