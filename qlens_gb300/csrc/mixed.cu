// mixed.cu -- mixed-precision inversion (placeholder until the tensor-core path lands).
#include "qlpix_ctx.h"
namespace qlpix {
int mixed_init(qlp_ctx* c) { (void)c; return QLP_OK; }
void mixed_free(qlp_ctx* c) { (void)c; }
int run_inversion_mixed(qlp_ctx* c, double regparam, cudaStream_t st, cudaEvent_t* ev)
{
    (void)c; (void)regparam; (void)st; (void)ev;
    set_error("%s (%d)", "mixed precision not available in this build", 0);
    return QLP_ERR_ARG;
}
}  // namespace qlpix
