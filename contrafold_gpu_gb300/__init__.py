"""contrafold_gpu_gb300: the CONTRAfold folding engine on GB300 (sm_103a).

Drop-in for the public API of `gpu_contrafold` (gpu_contrafold/__init__.py:17-31):

    from contrafold_gpu_gb300 import load, logZ_batch, sample_batch, mfe, mea, bpp
    P = load()                              # bundled CONTRAfold complementary params
    z = logZ_batch(["GGGGAAAACCCC"], P)     # log partition function(s), FP32
    structs = sample_batch(["GGGGAAAACCCC"], P, n_samples=10)
    db = mea("GGGGAAAACCCC", P, gamma=6)    # MEA structure
    prob = bpp("GGGGAAAACCCC", P)           # base-pair probabilities

Every compute call runs hand-written CUDA kernels through the C-ABI of
include/contrafold_gb300.h; there is no CPU fallback.
"""
from . import cpu, gpu
from .gpu import (bpp_batch, fold_tasks_gpu, logZ64_batch, logZ_batch, mea_batch, mfe_batch,
                  sample_batch)

load = cpu.load
cpu_logZ = cpu.logZ
mfe = cpu.mfe
mea = cpu.mea
bpp = cpu.bpp

__all__ = ["load", "cpu_logZ", "mfe", "mea", "bpp", "logZ_batch", "sample_batch", "fold_tasks_gpu",
           "cpu", "gpu", "mea_batch", "mfe_batch", "bpp_batch", "logZ64_batch"]
__version__ = "0.1.0"
