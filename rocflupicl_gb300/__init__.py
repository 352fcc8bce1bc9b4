"""rfgpu: a GB300-native residual engine for RocfluMP's unstructured
finite-volume Euler solver (WLSQ gradients + Venkatakrishnan limiter,
AUSM+/Roe/HLLC second-order fluxes, face-to-cell residual gather, Wray RK3
stage update with the perfect-gas EOS)."""
