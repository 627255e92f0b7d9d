// Version strings the reference's version.cmake would generate (oracle/_ref).
extern "C" {
const char* GIT_TAG = "reference sources, unmodified";
const char* GIT_REV = "built by oracle/ref/Makefile";
const char* GIT_BRANCH = "n/a";
}
