"""GB300-native engine for lyspeq's per-chunk quadratic maximum-likelihood step.

The compute path is the CUDA library ``liblqg.so`` (C ABI in include/lqg.h);
``lyspeq_gb300.lqg`` binds it, ``lyspeq_gb300.synth`` generates the seeded
synthetic workloads.
"""
__version__ = "0.1.0"
