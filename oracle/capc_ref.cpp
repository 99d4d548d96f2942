// capc_ref.cpp -- test infrastructure only.  Compiles the reference's cylinder-plane program
// (src/capc.cpp) unmodified from the reference tree, with its main() renamed, and
// exports its CasimirCP methods with C linkage so that tests/golden/make_golden_capc.py
// can record golden values.  Built by Makefile.ref into oracle/_ref/libcapc_ref.so;
// never linked into the product.
#define main capc_cli_main
#include "capc.cpp"
#undef main

// CasimirCP::logdet (capc.cpp:47-127): log det of the round trip at wave number q
extern "C" double capc_ref_logdet(double R, double d, int lmax, double q, char DN, int detalg)
{
    CasimirCP c(R, d, (detalg_t)detalg);
    c.set_lmax(lmax);
    return c.logdet(q, DN);
}

// CasimirCP::energy (capc.cpp:129-153): T = 0 energy per length in units of hbar c
extern "C" double capc_ref_energy(double R, double d, int lmax, char p, double epsrel, int detalg)
{
    CasimirCP c(R, d, (detalg_t)detalg);
    c.set_lmax(lmax);
    return c.energy(p, 0, epsrel);
}
