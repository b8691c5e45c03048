// Stand-in for the staged header of the same name (test infrastructure): see graphit_host.h.
#pragma once
#include "../graphit_host.h"
