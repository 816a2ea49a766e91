// gs_qdht_tc.cu -- placeholder until the tcgen05 kernel lands: mixed handles are refused.
#include "gs_qdht_tc.h"

namespace gs {
struct QdhtTc {};
QdhtTc* qdht_tc_create(int, int, cudaStream_t, std::string* msg) {
    if (msg) *msg = "mixed-precision QDHT not built";
    return nullptr;
}
int qdht_tc_set_matrix(QdhtTc*, const double*, const double*, std::string* msg) {
    if (msg) *msg = "not built";
    return 1;
}
cudaError_t qdht_tc_run(QdhtTc*, int, const float*, float*, const LstepArgs&, long long*, std::string* msg) {
    if (msg) *msg = "not built";
    return cudaErrorNotSupported;
}
void qdht_tc_destroy(QdhtTc*) {}
}  // namespace gs
