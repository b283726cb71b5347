"""GB300-native hot path of GLPhase's MH/HMM haplotype sampler.

The compute lives in a CUDA shared library (``libglphase_gpu.so``, built from
``glphase_gb300/csrc`` for sm_103a) behind the C ABI declared in
``include/glphase_gpu.h``.  This package holds the host-side mirror of the
reference's interface for that path:

* :mod:`glphase_gb300.model`   -- Insti::initialize's model constants
* :mod:`glphase_gb300.native`  -- ctypes binding of the C ABI (fails loudly
  when the library is missing)
* :mod:`glphase_gb300.hmmlike` -- HMMLike / HMMLikeCUDA mirror and the
  device-resident generation engine
* :mod:`glphase_gb300.synth`   -- seeded synthetic workloads
"""

__all__ = ["model", "synth"]
