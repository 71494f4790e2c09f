// placeholder: points and lines are added next
#include "swr_ops.h"
