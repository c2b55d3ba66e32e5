"""CPU oracle for the VHS RF decode hot path -- TEST INFRASTRUCTURE ONLY.

This package is a plain numpy/scipy restatement of the managed ``exact``
backend of vhs-decode-dotnet (VHSDecode.Core) for the RF path:
int16 RF -> band-pass/Hilbert -> FM demod -> video LPF/de-emphasis ->
pulses -> line locations -> hsync refinement -> sinc TBC -> uint16.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it, and only as the checker.  The product path (the C-ABI
library under ``vhs-decode-dotnet_gb300/``) never calls into it.

Parity pins: the sinc resampler is pinned against the platform-independent
SHA-256 golden vectors of ``tests/VHSDecode.Tests/TbcParallelResamplerTests.cs``
(see tests/golden/), the pulse state machine and spike repair against the
known answers in ``PulseDetectionReuseTests.cs`` / ``CompatibilityTests.cs``.
The block demodulator's own SHA-256 fixtures (``tape-family-v0.4.0.json``)
are asserted by the reference only on Windows and depend on its pocketfft
port's exact rounding, so block-level parity is pinned by the analytic
known-answer tests and by tolerance, not by hash.
"""
