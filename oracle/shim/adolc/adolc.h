#include "adouble.h"
#include "taping.h"
#include "drivers/drivers.h"
