"""
tvb_hpc on GB300: a drop-in for the network time step of tvb-hpc.

The model / coupling / scheme / network classes keep the attribute schema of
tvb-hpc (tvb_hpc/model.py, coupling.py, scheme.py, network.py), and
``transforms.network_time_step`` returns an executor with the same keyword
call convention as the generated loopy kernel
(tvb_hpc/examples/hackathon.py:48-54).  The executor and the engine in
``tvb_hpc.engine`` run hand-written sm_103a CUDA kernels through the ctypes
C ABI declared in include/tvbg.h; there is no CPU fallback.
"""

import logging
import os

__version__ = '0.1.0+gb300'

logging.getLogger('tvb_hpc').setLevel(
    getattr(logging, os.environ.get('TVB_LOG', 'INFO'), logging.INFO))
