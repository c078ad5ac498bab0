// hs_batch_api.cpp -- batched solver C ABI (filled in by the batched kernels).
#include "../../include/moose_gb300.h"
