#include "gsl_matrix_double.h"
