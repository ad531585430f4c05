/* placeholder, replaced below */
#include "pvvc_oracle.h"
