// Digamma table (netcalc/include/psi.h:160-163): psi has n+1 entries,
// psi[0] = 0, psi[1] = -0.57721566490153 (as float),
// psi[i+1] = psi[i] + (float)(1.0 / (float)i).
#ifndef NETSCI_GB300_NETCALC_PSI_H
#define NETSCI_GB300_NETCALC_PSI_H
#include "cuarray.h"
void generatePsi(CuArray<float>* psi, int n);
#endif
