"""Physical constants of the meV / T / ps / Angstrom unit system (core/include/utility/Constants.hpp)."""
import ctypes

from .spiritlib import fn

mu_B = fn("Constants_mu_B", [], ctypes.c_double)()
mu_0 = fn("Constants_mu_0", [], ctypes.c_double)()
k_B = fn("Constants_k_B", [], ctypes.c_double)()
hbar = fn("Constants_hbar", [], ctypes.c_double)()
gamma = fn("Constants_gamma", [], ctypes.c_double)()
g_e = fn("Constants_g_e", [], ctypes.c_double)()
pi = fn("Constants_Pi", [], ctypes.c_double)()
