/* empty: see mkl.h */
