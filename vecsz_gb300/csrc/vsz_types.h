// Internal shared definitions: re-exports the public C-ABI header (status codes, enums).
#pragma once
#include "../../include/vecsz_gb300.h"
