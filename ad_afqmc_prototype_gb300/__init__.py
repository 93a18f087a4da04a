"""GB300-native phaseless-AFQMC step engine (restricted walkers, RHF trial,
Cholesky Hamiltonian).  The module layout mirrors the reference package
ad_afqmc_prototype (core/, ham/, trial/, meas/, prop/, walkers.py); every
numerical operation runs in the CUDA library libafqmc_gb300.so through the
C ABI declared in include/afqmc_gb300.h."""

__version__ = "0.1.0"
