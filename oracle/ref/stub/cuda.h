/* empty stand-in: the reference includes this header but the CPU build of
   its kernels and host routines uses nothing from it */
#pragma once
