/* empty stand-in: the reference harness compiles kernels only */
#pragma once
