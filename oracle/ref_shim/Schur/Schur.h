// Empty stand-in: Mat-8.3.1/Mat.h includes Schur/Schur.h, which that snapshot does not ship.
