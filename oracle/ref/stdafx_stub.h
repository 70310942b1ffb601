/* stdafx.h stub: stands in for the reference's precompiled-header include
 * (which pulls in <stdio.h> and Windows headers).  The standard headers are
 * included here, before any reference header defines its min/max macros. */
#pragma once
#ifdef __cplusplus
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>
#include <queue>
#else
#include <stdio.h>
#endif
