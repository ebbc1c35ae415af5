/* Stand-in for the build configuration header the reference's build system
 * generates: the vendored levmar is compiled here without LAPACK (its own
 * LU solver), which for the one-parameter fit the split cross-validation
 * runs gives the same iterates as the LAPACK build up to rounding. */
