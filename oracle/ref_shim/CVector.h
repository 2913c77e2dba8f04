// The reference includes its own header under two spellings (CVector.h and
// cvector.h); on a case-sensitive file system this forwards the first.
#pragma once
#include "cvector.h"
