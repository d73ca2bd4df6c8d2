class Line2D:
    pass
