"""spirit_gb300: the spin-dynamics hot path of Spirit (LLG with dipolar FFT, batched
ensembles, GNEB) rebuilt for one NVIDIA GB300 (sm_103a).

The Python modules mirror the reference's `spirit` package (state, hamiltonian, geometry,
configuration, chain, transition, simulation, system, quantities, parameters.llg/gneb) on top of
the C API of libspirit_gb300.so.  `import spirit_gb300.state` loads the library and fails loudly
if it is not built -- there is no CPU fallback.
"""
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libspirit_gb300.so")
