// Own dense Hermitian eigensolver (tridiagonal reduction + bisection + inverse iteration).
#include "bse_internal.h"

namespace bse {

int own_heevd(bse_ctx* c, int n, void* dA, int lda, bool fp64, double* dW, bool vectors) {
    (void)n; (void)dA; (void)lda; (void)fp64; (void)dW; (void)vectors;
    return fail(c, BSE_ERR_BAD_INPUT, "own eigensolver not available in this build");
}

}  // namespace bse
