"""GB300-native Bethe-Salpeter solver (q->0 Tamm-Dancoff BSE: kernel build, dense
Hermitian eigensolve, oscillator strengths and eps2) behind the C ABI of
include/bse_gpu.h.  The package directory name is not a Python identifier, so it is
loaded under the alias ``bse_gb300`` (see ``load_package`` in __graft_entry__)."""
from . import constants, model, synth, capi, w90io  # noqa: F401
# gpu (ctypes binding) and adjoint (torch) are imported on demand
