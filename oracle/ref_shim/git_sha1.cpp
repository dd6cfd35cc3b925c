// Stand-in for the source the reference's CMake configures from
// cmake/git_sha1.cpp.in (the git state recorded in its reports).
extern const char g_GIT_SHA1[] = "unknown";
extern const char g_GIT_LOCAL_CHANGES_STATUS[] = "unknown";
extern const char g_GIT_REFSPEC[] = "unknown";
