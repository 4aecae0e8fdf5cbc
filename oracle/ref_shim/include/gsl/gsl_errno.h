#include "ref_gsl.h"
