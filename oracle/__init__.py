"""CPU restatement of the SaclayMocks hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker the CUDA library is compared against, and the timed
CPU baseline of ``bench.py``.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference arm of ``bench.py`` may import it; the product package
``saclaymocks_gb300`` never does (its CUDA path fails loudly instead of falling back).

Every function cites the reference file:line it restates (paths inside
igmhub/SaclayMocks).  Parity of this restatement is pinned against the golden
fixtures of ``tests/golden`` (made by running the reference's own functions); the
FFT library of the reference (FFTW through pyfftw) is absent here, so FFT results are
pinned through numpy's pocketfft only.

Modules: ``grf`` (make_boxes), ``skewers`` (make_spectra read + merge_spectra small
scales + FGPA), ``p1d`` (P1D estimator, binned reductions), ``fit`` (the (a,b,c)
loss and its gradients), ``fgpa_pdf`` (analytic <F>), ``cskewers`` (the C
restatement of the trilinear read + FGPA, multi-threaded, used as CPU baseline).
"""
