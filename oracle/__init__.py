"""CPU oracle for the q-SFT hot path -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

This package restates, in plain numpy / Python, the reference algorithm of
basics-lab/qsft for the path the CUDA library accelerates: coset query
generation, synthetic-signal evaluation, the q-ary GWHT, bin-domain noise,
singleton detection (noiseless, NSO "nso1", Reed-Solomon coded source) and the
peeling loop.  Every function cites the reference file:line it follows.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import it, and only as the checker or the timed CPU baseline.  The
``qsft_gb300`` package never imports it; it fails loudly when its CUDA library
is missing instead of falling back to this code.

Pinning: ``tests/test_oracle_golden.py`` checks this restatement against
fixtures produced by running the reference itself (``tests/golden/``).  The
Reed-Solomon part is NOT pinned against the reference: the reference delegates
it to ``galois==0.1.1`` (numba-JIT ``decode_jit``), which is not installed, so
``oracle.rs`` restates the published algorithms (Berlekamp-Massey, Chien
search, Forney) and is checked by encode->syndrome->decode round trips and by
ground-truth support recovery -- parity unpinned for that part.
"""
from .qsft_oracle import *  # noqa: F401,F403
from . import rs  # noqa: F401
