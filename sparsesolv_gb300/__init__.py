"""GB300-native Krylov hot path of SparseSolv (shifted IC(0), ICCG, IC-MRTR,
Eisenstat SGS-MRTR; real and complex-symmetric), behind the reference's API."""
