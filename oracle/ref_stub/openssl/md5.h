/* Empty stand-in: include/kokkos_md5.hpp includes <openssl/md5.h> but calls
 * nothing from it. */
#pragma once
