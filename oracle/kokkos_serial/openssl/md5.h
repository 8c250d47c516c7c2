// openssl/md5.h -- empty stand-in: the reference includes it, but the code
// compiled for the tests uses its own MD5 (include/kokkos_md5.hpp).  Test
// infrastructure only.
#pragma once
