#pragma once
#include "../EleFits/FitsFile.h"
