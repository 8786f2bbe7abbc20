// Stand-in: the definitions live in palabos3D.h (reference harness only).
