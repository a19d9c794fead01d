#pragma once
#include "FitsFile.h"
