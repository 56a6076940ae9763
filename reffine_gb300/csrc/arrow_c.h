#pragma once
#include "reffine_gb300/arrow_c.h"
