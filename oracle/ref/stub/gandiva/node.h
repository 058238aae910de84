#pragma once
#include "gandiva_stub.h"
