// Forwarding header of the VIGRA shim (test oracle only).
#pragma once
#include "vigra_shim.hxx"
