"""GB300-native 3D FDTD solver: a drop-in replacement for the Yee time step of ravelec/FDTD."""
