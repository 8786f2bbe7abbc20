// Stand-in: dynamicsTemplates is declared in palabos3D.h (reference harness only).
