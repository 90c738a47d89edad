// case_parser.cpp -- placeholder replaced below
#include "hystrath_gb300.h"
extern "C" int dsmc_parse_case(const char*, dsmc_case_spec*) { return DSMC_ERR_IO; }
extern "C" int dsmc_create(const char*, dsmc_handle** out) { *out = nullptr; return DSMC_ERR_IO; }
