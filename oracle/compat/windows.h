/* Empty stand-in for <windows.h>.
 *
 * TEST INFRASTRUCTURE ONLY.  src/properties.cpp of the reference includes
 * <windows.h> but uses nothing from it; this file lets g++ on Linux compile
 * that reference source unmodified for the parameter golden fixtures. */
