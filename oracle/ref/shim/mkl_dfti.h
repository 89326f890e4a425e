/* MKL DFTI stand-in: included by the reference FFT header, never used on the sine path. */
