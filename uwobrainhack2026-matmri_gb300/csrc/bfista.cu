// placeholder: replaced by the bfista / powermethod implementation
#include "sense.cuh"
using namespace mmr;
extern "C" int mmr_powermethod(mmr_sense*, const void*, int32_t, double, double*, double*, void*) {
    return guarded([&] { MMR_THROW(MMR_ERR_UNSUPPORTED, "powermethod not built yet"); });
}
extern "C" int mmr_bfista_solve(mmr_sense*, const void*, const int32_t*, const float*, int32_t, const void*,
                                const mmr_bfista_opts*, void*, mmr_bfista_hist*, void*) {
    return guarded([&] { MMR_THROW(MMR_ERR_UNSUPPORTED, "bfista not built yet"); });
}
