/* stub: nothing from the GL helpers is used by the pinned kernels */
#pragma once
