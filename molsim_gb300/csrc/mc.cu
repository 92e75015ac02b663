// mc.cu — Monte Carlo trial-move energy differences (rows A13, A14).
#include "mg_internal.cuh"

int mg_mc_init(mg_handle *h) { (void)h; return MG_OK; }
int mg_mc_after_utotal(mg_handle *h) { (void)h; return MG_OK; }
int mg_mc_dutotal(mg_handle *h, int, const int32_t *, const double *, double *, double *, double *, int32_t *) {
    return mg_fail(h, MG_ERR_UNSUPPORTED, "DUTotal is not built yet");
}
int mg_mc_accept(mg_handle *h) { return mg_fail(h, MG_ERR_UNSUPPORTED, "not built yet"); }
int mg_mc_batch(mg_handle *h, int, const int32_t *, const double *, double *, int32_t *) {
    return mg_fail(h, MG_ERR_UNSUPPORTED, "not built yet");
}
