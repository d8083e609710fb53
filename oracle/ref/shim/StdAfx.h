/* Case alias for a case-sensitive filesystem: the reference includes "StdAfx.h" but ships "stdafx.h". */
#pragma once
#include "stdafx.h"
