"""Generate tests/golden/transforms.npz: FFTW-definition transform vectors.

FEN's Poisson solvers call FFTW 3.3.10 (dft_r2c_1d, dft_c2r_1d, dft_1d, r2r_1d with
REDFT10/REDFT01; src/poisson.f90:148-169, 272-275, 635-674, 801-822, 888-909).  FFTW is not
in this image, so these vectors come from independent implementations of the same published
definitions: numpy.fft (pocketfft) for the DFTs and scipy.fft.dct types 2 and 3 (which equal
REDFT10 and REDFT01 unnormalised).  Inputs are seeded; sizes cover the radix-2/3 lengths
the solvers use.

    python tests/golden/make_golden.py
"""
import os

import numpy as np
import scipy.fft as sf

SIZES = [8, 12, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512]


def main():
    rng = np.random.Generator(np.random.PCG64(20241203))
    out = {}
    for n in SIZES:
        x = rng.standard_normal(n)
        z = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        X = np.fft.rfft(x)
        out[f"x_{n}"] = x
        out[f"z_{n}"] = z
        out[f"fft_{n}"] = np.fft.fft(z)
        out[f"bfft_{n}"] = np.fft.ifft(z) * n          # FFTW_BACKWARD, unnormalised
        out[f"r2c_{n}"] = X
        out[f"c2r_{n}"] = np.fft.irfft(X, n) * n       # unnormalised c2r of r2c(x) = n x
        out[f"redft10_{n}"] = sf.dct(x, type=2)
        out[f"redft01_{n}"] = sf.dct(x, type=3)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "transforms.npz")
    np.savez_compressed(path, **out)
    print(path)


if __name__ == "__main__":
    main()
