"""Physical constants and flag values shared by the host code and the tests.

The numbers restate bse.version13.cpp:28-33 (minval, pigreco, conversion_parameter)
and the enums of include/bse_gpu.h.
"""
import math

MINVAL = 1.0e-5                               # bse.version13.cpp:28
PI = math.pi                                  # bse.version13.cpp:29 (pigreco)
CONV = (1.602176634 * 1000) / 8.8541878176    # e/eps0 in eV*Angstrom, bse.version13.cpp:32
INV_EPS_EMPIRICAL = 0.086206897               # bse.version13.cpp:2697 (1/11.6, silicon)

# include/bse_gpu.h enums
BSE_V_BARE_3D, BSE_V_BARE_2D = 0, 1
BSE_W_EMPIRICAL, BSE_W_RYTOVA_KELDYSH, BSE_W_BARE, BSE_W_RPA = 0, 1, 2, 3
BSE_FP64, BSE_MIXED = 0, 1
BSE_EIG_OWN, BSE_EIG_CUSOLVER = 0, 1

STATUS = {
    0: "BSE_OK",
    -1: "BSE_ERR_BAD_INPUT",
    -2: "BSE_ERR_NO_DEVICE",
    -3: "BSE_ERR_OOM",
    -4: "BSE_ERR_NOT_CONVERGED",
    -5: "BSE_ERR_CUDA",
    -6: "BSE_ERR_STATE",
}
