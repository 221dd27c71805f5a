// TEST INFRASTRUCTURE: HDF5 I/O is not used by the solver sources.
#pragma once
