/*
 * rt_exception.h: exception type thrown by the host engine API.
 *
 * The reference reports errors from constructors and allocators by throwing
 * rt_Exception carrying a message (core/system/system.h:175-190); the GB300
 * host keeps that behaviour, converting non-zero C-ABI statuses into it.
 */
#ifndef QR_RT_EXCEPTION_H
#define QR_RT_EXCEPTION_H

class rt_Exception
{
public:
    const char *err;
    explicit rt_Exception(const char *e) : err(e) {}
};

#endif /* QR_RT_EXCEPTION_H */
