/*
 * version.h — build version of the GB300 decoder, under the macro names the
 * reference's main.cpp prints (version.h: VERSION_STR, VERSION_STR3).
 */
#ifndef H264R_COMPAT_VERSION_H
#define H264R_COMPAT_VERSION_H

#define MAJOR_VERSION   1
#define MINOR1_VERSION  0
#define MINOR2_VERSION  0
#define MINOR3_VERSION  0

#define VERSION_STR     MAJOR_VERSION.MINOR1_VERSION.MINOR2_VERSION.MINOR3_VERSION
#define VERSION_STR2(S) #S
#define VERSION_STR3(S) VERSION_STR2(S)

#endif /* H264R_COMPAT_VERSION_H */
