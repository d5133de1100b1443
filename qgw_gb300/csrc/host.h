// host.h -- host helpers shared by the C ABI implementation.
#pragma once
#include "../../include/qgw_gpu.h"

double qgw_host_nu_hyper(const qgw_params* p);
double qgw_host_wind(const qgw_params* p, int j);
