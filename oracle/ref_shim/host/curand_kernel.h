/* Host-only build of the reference hash helpers: cuRAND device state is not
 * used (cu_random is 0 in GPU/dyhash/dy_hash.h:50). */
#pragma once
