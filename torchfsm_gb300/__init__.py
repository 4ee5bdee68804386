"""GB300-native Fourier-spectral ETD time stepping with the torchfsm API."""
