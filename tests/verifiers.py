"""placeholder"""
def install():
    pass
