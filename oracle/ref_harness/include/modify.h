// Stand-in (reference harness only).
