"""mptc_gb300: the MPTC encoder hot path on GB300 (sm_103a) behind a C ABI.

Modules: ``encoder`` (per-stream encoder), ``batch`` (many streams per call),
``model`` / ``training`` (learned candidate proposal), ``stream`` (MPTC
stream writer and reader), ``decoder`` (GPU decode and endpoint transform),
``synth`` (seeded synthetic frames). The work runs in ``libmptc_gb300.so``
(CUDA) and ``libmptc_host.so`` (stream container and arithmetic coder); there
is no CPU fallback for any GPU step.
"""
