import hashlib

import numpy as np


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def unhex(xs):
    return np.array([float.fromhex(x) for x in xs])


def kernel_macros():
    """The integer #defines of include/dvmh_gb_kernels.h (variant counts and
    numbers), evaluated in order: the tests follow the header."""
    import os
    import re
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "dvmh_gb_kernels.h")
    env = {}
    for line in open(path):
        m = re.match(r"#define\s+(DVMHGB_\w+)\s+(.+?)\s*(/\*.*)?$", line)
        if not m:
            continue
        try:
            env[m.group(1)] = int(eval(m.group(2), {}, dict(env)))
        except Exception:
            pass
    return env


J3 = kernel_macros()
J3_STENCILS = J3["DVMHGB_JAC3D_VARIANTS"]      # stencil variants
J3_FUSED = J3["DVMHGB_JAC3D_FUSED_VARIANTS"]   # variants of the fused pair
J3_IN_PLACE = (J3["DVMHGB_JAC3D_UNFUSED"], J3["DVMHGB_JAC3D_OVERLAP"], J3["DVMHGB_JAC3D_OVERLAP_Q"])
J3_ONE_PASS_Q = [J3["DVMHGB_JAC3D_FUSED_Q"], J3["DVMHGB_JAC3D_FUSED_Q"] + 1,
                 J3["DVMHGB_JAC3D_FUSED_T"], J3["DVMHGB_JAC3D_FUSED_T"] + 1]
J3_STNUPD = J3["DVMHGB_JAC3D_STNUPD_VARIANTS"]  # variants of the cross-step pass
