// Empty stand-in: Mat-8.3.1/Mat.h includes EVD/EVD_Q.h, which that snapshot does not ship.
