// host.h -- host helpers shared by the C ABI implementation.
#pragma once
#include "../../include/qgw_gpu.h"

double qgw_host_nu_hyper(const qgw_params* p);
double qgw_host_wind(const qgw_params* p, int j);
#include <vector>
// The stochastic forcing's ring (init_stoch_forc, src/forcing.h:128-151):
// appends the (i, j) of the forced half-spectrum entries of the NX x NX
// transform to ij and returns their number N_P (0 when k_f == 0).
int qgw_host_forcing_ring(const qgw_params* p, std::vector<int>* ij);
